"""Host-side parts of the learned warm start (kevernals_gb300/warmstart.py):
training crops, chest-DT columns, phantom windows, masked targets and the
MLEM stopping / acceptance logic (driven by a fake plan)."""
import numpy as np
import pytest

from kevernals_gb300 import phantom as ph
from kevernals_gb300 import warmstart as ws
from kevernals_gb300.geometry import config_chest

torch = pytest.importorskip("torch")


def test_chest_crops_are_seeded_full_thickness_windows():
    s = torch.arange(8 * 64 * 96, dtype=torch.float32).reshape(8, 64, 96)
    x = -s
    a = ws.chest_crops(s, x, 32, 16, 5, seed=11)
    b = ws.chest_crops(s, x, 32, 16, 5, seed=11)
    assert len(a) == 5
    for (s1, x1), (s2, x2) in zip(a, b):
        assert s1.shape == (8, 16, 32) and torch.equal(s1, s2) and torch.equal(x1, -s1)
        flat = int(s1[0, 0, 0])
        y0, x0 = (flat // 96) % 64, flat % 96
        assert 0 <= x0 <= 96 - 32 and 0 <= y0 <= 64 - 16
        assert torch.equal(s1, s[:, y0:y0 + 16, x0:x0 + 32])
    assert any(not torch.equal(p[0], q[0]) for p, q in zip(a, ws.chest_crops(s, x, 32, 16, 5, seed=12)))


def test_column_geometry_uses_the_chest_grids():
    chest = config_chest()
    for seed in (ph.seed_for(5, 0), ph.seed_for(5, 7)):
        g, (cx, cy) = ws.column_geometry(ws.column_centre(seed), 128, 256)
        assert (g.nx, g.ny, g.nz) == (128, 256, chest.nz)
        # the column's voxel centres are chest voxel centres
        assert abs(cx / chest.dx - round(cx / chest.dx)) < 1e-6
        assert abs(cy / chest.dy - round(cy / chest.dy)) < 1e-6
        # sources are the chest's, moved into the column frame
        assert np.allclose(g.src, chest.src - np.array([cx, cy, 0.0], np.float32), atol=1e-3)
        # per-view detector ROIs lie on the chest's pixel grid, inside its detector
        off = (g.det_origin[:, :2] + np.array([cx, cy], np.float32)) - chest.det_origin[:, :2]
        pix = off / np.array([chest.du, chest.dv], np.float32)
        assert np.allclose(pix, np.round(pix), atol=1e-2)
        assert (np.round(pix) >= 0).all()
        assert (np.round(pix[:, 0]) + g.nu <= chest.nu).all() and (np.round(pix[:, 1]) + g.nv <= chest.nv).all()


def test_window_params_shift_the_chest_phantom():
    off = (12.4, -8.0, 0.0)
    w = ws.window_params(ph.seed_for(5, 3), off, n_ellipsoids=10)
    full = ph.ellipsoid_params(1024, 1024, 128, 0.4, 0.4, 2.5, 10, ph.seed_for(5, 3))
    assert np.allclose(w[:, 0:3] + np.asarray(off, np.float32), full[:, 0:3])
    assert np.array_equal(w[:, 3:], full[:, 3:])


def test_mask_margin_only_blanks_the_lateral_margin():
    x = torch.ones(4, 40, 50)
    t = ws.mask_margin(x, margin=3)
    inner = t[:, 3:-3, 3:-3]
    assert not torch.isnan(inner).any()
    assert int(torch.isnan(t).sum()) == 4 * (40 * 50 - 34 * 44)
    assert torch.equal(x, torch.ones(4, 40, 50))          # the input is untouched


class FakePlan:
    """Stands in for engine.Plan.mlem: reports a fixed residual sequence to
    the callback, one value per iteration, as kv_mlem does."""

    def __init__(self, residuals):
        self.residuals = residuals
        self.updates = 0

    def mlem(self, p, x, iters, callback=None):
        for it in range(iters):
            if callback(it, self.residuals[it], 0.0):
                return
            self.updates += 1


def test_iterations_to_residual_counts_updates_and_rejects_bad_starts():
    res = [1.0, 0.5, 0.3, 0.2, 0.15, 0.1]
    plan = FakePlan(res)
    n, r = ws.iterations_to_residual(plan, None, None, target=0.2, max_iters=10)
    assert (n, r) == (3, 0.2) and plan.updates == 3
    plan = FakePlan(res)
    n, r, r0, rejected = ws.iterations_to_residual(plan, None, None, 0.2, 10, reject_above=0.9)
    assert rejected and (n, r0) == (0, 1.0) and plan.updates == 0
    plan = FakePlan(res)
    n, r, r0, rejected = ws.iterations_to_residual(plan, None, None, 0.2, 10, reject_above=2.0)
    assert not rejected and (n, r, r0) == (3, 0.2, 1.0)
    plan = FakePlan(res)
    n, r = ws.iterations_to_residual(plan, None, None, target=0.01, max_iters=4)
    assert (n, r) == (4, 0.15) and plan.updates == 4
