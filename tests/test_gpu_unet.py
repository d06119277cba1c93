"""The U-Net warm start: forward and gradients of the tensor-core kernels
against an FP64 PyTorch reference, training progress, checkpoint round trip."""
import numpy as np
import pytest

from kevernals_gb300 import build, engine

import unet_torch_ref as ref

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    build.build()
    return engine.Context(0)


def smooth_input(shape, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.rand(shape, generator=g, dtype=torch.float64)
    x = torch.nn.functional.avg_pool3d(x[None, None], 3, stride=1, padding=1)[0, 0]
    return x.float().numpy()


def perturbed(net, seed):
    """Random non-zero output layer so every layer's gradient is exercised."""
    st, step = net.get_state()
    n = net.num_params
    lay = ref.layout()
    rng = np.random.default_rng(seed)
    st[lay["w_out"]:lay["w_out"] + 16] = rng.normal(0, 0.3, 16)
    net.set_state(st, step)
    return st[:n].copy()


def test_parameter_layout_matches(ctx):
    net = engine.UNet(ctx, seed=1)
    assert net.num_params == ref.layout()["n"]


def test_forward_matches_fp64_reference(ctx):
    net = engine.UNet(ctx, seed=2)
    params = perturbed(net, 2)
    x = smooth_input((16, 16, 128), 0)
    y = net.forward(x)
    yr = ref.forward(torch.from_numpy(x).double(), params).numpy()
    d = y - x
    dr = yr - x
    err = np.linalg.norm(d - dr) / np.linalg.norm(dr)
    print(f"U-Net forward vs FP64 reference (BF16-rounding emulated): rel L2 of f(x) {err:.2e}")
    assert err < 2e-2


def test_gradients_match_fp64_reference(ctx):
    net = engine.UNet(ctx, seed=3)
    params = perturbed(net, 3)
    x = smooth_input((16, 16, 128), 1)
    t = x * 0.7 + 0.05
    loss, g = net.gradients(x, t)
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    yr = ref.forward(torch.from_numpy(x).double(), ref.unpack(p))
    lr = ((yr - torch.from_numpy(t).double()) ** 2).mean()
    lr.backward()
    gr = p.grad.numpy()
    assert loss == pytest.approx(lr.item(), rel=1e-2)
    lay = ref.layout()
    blocks = [("first", lay["w_first"], 432)] + \
             [(f"conv{i}", w, co * 27 * cin) for i, (cin, co, w, b) in enumerate(lay["convs"])] + \
             [("out", lay["w_out"], 16)]
    worst = 0.0
    for name, o, n in blocks:
        e = np.linalg.norm(g[o:o + n] - gr[o:o + n]) / max(np.linalg.norm(gr[o:o + n]), 1e-30)
        worst = max(worst, e)
        assert e < 8e-2, (name, e)
    cos = float(np.dot(g, gr) / (np.linalg.norm(g) * np.linalg.norm(gr)))
    print(f"U-Net gradients vs FP64 autograd: worst layer rel L2 {worst:.2e}, cosine {cos:.6f}")
    assert cos > 0.998


def test_training_reduces_loss_and_checkpoint_roundtrip(ctx, tmp_path):
    net = engine.UNet(ctx, seed=4)
    x = smooth_input((16, 32, 128), 2)
    t = np.ascontiguousarray(0.5 * x + 0.1 * np.roll(x, 1, axis=2), np.float32)
    losses = [net.train_step(x, t, lr=1e-3) for _ in range(60)]
    print(f"U-Net training: loss {losses[0]:.4e} -> {losses[-1]:.4e} in 60 Adam steps")
    assert losses[-1] < 0.5 * losses[0]
    net.save(tmp_path / "ckpt.npz")
    y1 = net.forward(x)
    other = engine.UNet(ctx, seed=99)
    other.load(tmp_path / "ckpt.npz")
    assert np.array_equal(other.forward(x), y1)
    # resumed training continues identically
    l_a = net.train_step(x, t, lr=1e-3)
    l_b = other.train_step(x, t, lr=1e-3)
    assert l_a == l_b
