"""Every convolution shape of the U-Net, one layer at a time, through the C ABI
(kv_conv3_bf16): the tcgen05 / TMA implicit GEMM against the mma.sync kernel
(the same products summed in the same K order: bit-identical) and against an
FP64 conv3d of the same BF16 inputs and weights.  Against FP64 the output
differs by the final rounding to BF16 (half an ulp) plus the error of the
FP32 accumulation on the tensor cores, which align the products of each MMA
step to the largest and truncate: measured 1e-6 .. 6e-6 absolute on sums of
5184 products whose magnitudes add to ~50, so the bound is
2^-8 |ref| + 2^-20 sum|w x|, and at least 99 % of the outputs must equal
the FP64 value rounded to nearest even."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (level, c1, c2, cout, relu) at a 16 x 32 x 128 input (level l: each side
# halved l times): the encoder, the bottleneck, the decoder's concatenated
# inputs (upsampled ++ skip) and the backward-data convolutions (transposed
# weights: c_out = the forward layer's input channels)
SHAPES = [
    (0, 16, 0, 16, True), (1, 16, 0, 32, True), (1, 32, 0, 32, True), (2, 32, 0, 64, True),
    (2, 64, 0, 64, True), (3, 64, 0, 128, True), (3, 128, 0, 128, True),
    (2, 128, 64, 64, True), (1, 64, 32, 32, True), (0, 32, 16, 16, True),
    (3, 128, 0, 64, False), (2, 64, 0, 192, False), (1, 32, 0, 96, False), (0, 16, 0, 48, False),
]
BASE = (16, 32, 128)


def _bf16_bits(x):
    """float32 array -> BF16 bit patterns (round to nearest even) and their float32 values."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r, (r.astype(np.uint32) << 16).view(np.float32)


def _conv(ctx, a, c1, b, c2, w, bias, relu, cout, dims, kernel):
    import torch
    from kevernals_gb300 import _lib
    D, H, W = dims
    dev = torch.device("cuda")
    ta = torch.from_numpy(a.view(np.int16)).to(dev)
    tb = torch.from_numpy(b.view(np.int16)).to(dev) if c2 else None
    tw = torch.from_numpy(w.view(np.int16)).to(dev)
    tbias = torch.from_numpy(bias).to(dev)
    out = torch.empty((D, H, W, cout), dtype=torch.int16, device=dev)
    ctx.use_torch_stream()
    st = _lib.lib().kv_conv3_bf16(ctx.handle, C.c_void_p(ta.data_ptr()), c1,
                                  C.c_void_p(tb.data_ptr() if tb is not None else 0), c2,
                                  C.c_void_p(tw.data_ptr()), C.c_void_p(tbias.data_ptr()), int(relu),
                                  C.c_void_p(out.data_ptr()), cout, D, H, W, kernel)
    assert st == 0, ctx.last_error()
    ctx.sync()
    return out.cpu().numpy().view(np.uint16)


@pytest.fixture(scope="module")
def ctx():
    from kevernals_gb300 import build, engine
    build.build()
    return engine.Context(0)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"L{s[0]}_{s[1]}+{s[2]}to{s[3]}" for s in SHAPES])
def test_conv_layer_tcgen05_vs_mma_sync_and_fp64(ctx, shape):
    torch = pytest.importorskip("torch")
    import torch.nn.functional as F
    lvl, c1, c2, cout, relu = shape
    dims = tuple(d >> lvl for d in BASE)
    D, H, W = dims
    rng = np.random.default_rng(lvl * 1000 + c1 * 7 + c2 * 3 + cout)
    a, af = _bf16_bits(rng.standard_normal((D, H, W, c1)).astype(np.float32))
    b, bf = _bf16_bits(rng.standard_normal((D, H, W, max(c2, 1))).astype(np.float32))
    cin = c1 + c2
    scale = 1.0 / np.sqrt(27 * cin)
    w, wf = _bf16_bits((rng.standard_normal((cout, 27, cin)) * scale).astype(np.float32))
    bias = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    tc = _conv(ctx, a, c1, b, c2, w, bias, relu, cout, dims, 1)
    ms = _conv(ctx, a, c1, b, c2, w, bias, relu, cout, dims, 2)
    assert np.array_equal(tc, ms)
    # FP64 reference on the same BF16 values
    x = af if c2 == 0 else np.concatenate([af, bf], axis=3)
    xt = torch.from_numpy(x.astype(np.float64)).permute(3, 0, 1, 2)[None]
    wt = torch.from_numpy(wf.astype(np.float64)).permute(0, 2, 1).reshape(cout, cin, 3, 3, 3)
    ref = F.conv3d(xt, wt, torch.from_numpy(bias.astype(np.float64)), padding=1)
    mag = F.conv3d(xt.abs(), wt.abs(), torch.from_numpy(np.abs(bias).astype(np.float64)), padding=1)
    if relu:
        ref = F.relu(ref)
    ref = ref[0].permute(1, 2, 3, 0).numpy()
    mag = mag[0].permute(1, 2, 3, 0).numpy()
    got = (tc.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    err = np.abs(got - ref)
    bound = 2 ** -8 * np.abs(ref) + 2 ** -20 * mag
    worst = np.unravel_index(np.argmax(err - bound), err.shape)
    assert np.all(err <= bound), (worst, got[worst], ref[worst], mag[worst])
    _, rne = _bf16_bits(ref.astype(np.float32))
    assert np.mean(got == rne) > 0.99
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 4e-3
