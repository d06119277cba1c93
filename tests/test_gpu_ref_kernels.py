"""The engine's RC kernels against the reference's own CUDA kernels, run on
the same GPU.

oracle/build_ref.sh compiles CudaPerformProjection and
CudaPerformBackProjection (Projector.cu:227-785) from the reference tree
into two cubins: with nvcc's defaults, as the reference ships them, and with
-fmad=false.  The engine's RC operators (kv_rc.cu, built with -fmad=false)
must match the -fmad=false build bit for bit, and the shipped build within
1e-5 relative L2 (the only difference is the multiply-add contraction the
shipped build allows) -- except the backprojector at the chest-DT geometry:
there the oblique footprint of a 2.5 mm slice (7-10 pixels of 0.2 mm)
overflows the reference's 11 x 11 pixel window, whose position is a
truncated float (Projector.cu:607-608), so a rounding change of the
intersection point can move the window by a pixel and change which pixels
enter the normalised mean.  The reference's two builds differ there by
~1e-2 relative L2 between themselves; the bound for that case is 2e-2.

Geometries: every ray must cross the volume's bottom and top faces (the
reference forward kernel has no defined result for a ray that misses the
volume, Projector.cu:79-85), so the detector is a central ROI:
  - the config-1 volume (256x256x64, 0.5x0.5x1.0 mm), 15 views over +-15 deg,
    224x224 pixels of 0.4 mm;
  - the chest-DT volume (1024x1024x128, 0.4x0.4x2.5 mm), views 0, 20, 40 and
    59 of the 60-view +-17.5 deg sweep, 256x256 pixels of 0.2 mm.

The cubins are built only where the reference tree is present; without them
these tests skip.
"""
import numpy as np
import pytest

from kevernals_gb300 import build, engine, phantom as ph
from kevernals_gb300.geometry import linear_sweep
from oracle import ref_gpu

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

REL_L2_SHIPPED = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def geom(name):
    if name == "config1-roi":
        return linear_sweep(256, 256, 64, 0.5, 0.5, 1.0, 15, 224, 224, 0.4, 0.4, 15.0)
    g = linear_sweep(1024, 1024, 128, 0.4, 0.4, 2.5, 60, 256, 256, 0.2, 0.2, 17.5)
    return g.subset_views([0, 20, 40, 59])


CASES = {"config1-roi": (40, 1), "chest-roi-4views": (400, 2)}
# relative L2 bound against the shipped (multiply-add contracting) build
BACK_SHIPPED = {"config1-roi": REL_L2_SHIPPED, "chest-roi-4views": 2e-2}


@pytest.fixture(scope="module")
def ctx():
    if not (ref_gpu.available("fma") and ref_gpu.available("nofma")):
        pytest.skip("reference kernels not compiled (oracle/build_ref.sh needs the reference tree)")
    build.build()
    c = engine.Context(0)
    c.use_torch_stream()
    return c


def phantom(ctx, g, name):
    n, cfg = CASES[name]
    params = ph.ellipsoid_params(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, n, ph.seed_for(cfg, 7))
    return engine.phantom(ctx, g, params, device=True)


@pytest.mark.parametrize("name", list(CASES))
def test_rc_forward_matches_reference_kernel(ctx, name):
    g = geom(name)
    assert ref_gpu.all_rays_cross_volume(g)
    vol = phantom(ctx, g, name)
    ref = ref_gpu.forward(g, vol, variant="fma").cpu().numpy()
    ref_nofma = ref_gpu.forward(g, vol, variant="nofma").cpu().numpy()
    plan = engine.Plan(ctx, g, "rc")
    ours = plan.forward(vol)
    torch.cuda.synchronize()
    ours = ours.cpu().numpy()
    plan.close()
    err = rel_l2(ours, ref)
    print(f"{name}: RC forward vs reference kernel: rel L2 {err:.3e} (shipped build), "
          f"{int(np.count_nonzero(ours != ref_nofma))} of {ours.size} differ from the -fmad=false build")
    np.testing.assert_array_equal(ours, ref_nofma)
    assert err <= REL_L2_SHIPPED


@pytest.mark.parametrize("name", list(CASES))
def test_rc_back_matches_reference_kernel(ctx, name):
    g = geom(name)
    vol = phantom(ctx, g, name)
    plan = engine.Plan(ctx, g, "rc")
    proj = plan.forward(vol)
    torch.cuda.synchronize()
    ref = ref_gpu.back(g, proj, variant="fma").cpu().numpy()
    ref_nofma = ref_gpu.back(g, proj, variant="nofma").cpu().numpy()
    ours = plan.back(proj)
    torch.cuda.synchronize()
    ours = ours.cpu().numpy()
    plan.close()
    err = rel_l2(ours, ref)
    print(f"{name}: RC back vs reference kernel: rel L2 {err:.3e} (shipped build), "
          f"{int(np.count_nonzero(ours != ref_nofma))} of {ours.size} differ from the -fmad=false build")
    np.testing.assert_array_equal(ours, ref_nofma)
    assert err <= BACK_SHIPPED[name]


def test_reference_forward_refuses_missing_rays():
    """A geometry with rays that miss the volume is refused on the host; the
    kernel is never launched on it."""
    g = linear_sweep(256, 256, 64, 0.5, 0.5, 1.0, 15, 512, 512, 0.4, 0.4, 15.0)
    assert not ref_gpu.all_rays_cross_volume(g)
    with pytest.raises(ValueError):
        ref_gpu.forward(g, torch.zeros(g.volume_shape, device="cuda"))
