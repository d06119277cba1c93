"""FP64 PyTorch (CPU) reference of the kvtomo U-Net, for the tests.

Same architecture and flat parameter layout as kevernals_gb300/csrc/kv_unet.cu:
first conv w[16][27] + b[16]; then 13 conv layers, each W[cout][27][cin]
(tap = kz*9 + ky*3 + kx) + b[cout], every block start rounded up to a multiple
of 8 floats; output layer w[16] + b[1] (then padding to 8).  The rounding of
the BF16 tensors the kernels store (3x3x3 conv weights, activations, pool
outputs) is emulated so that the remaining difference is FP32 accumulation.
"""
import torch
import torch.nn.functional as F

SPEC = [(16, 0, 16), (16, 0, 32), (32, 0, 32), (32, 0, 64), (64, 0, 64), (64, 0, 128), (128, 0, 128),
        (128, 64, 64), (64, 0, 64), (64, 32, 32), (32, 0, 32), (32, 16, 16), (16, 0, 16)]


def layout():
    off = 0
    lay = {"w_first": off}
    off += 16 * 27
    lay["b_first"] = off
    off += 16
    convs = []
    for c1, c2, co in SPEC:
        w = off
        off += co * 27 * (c1 + c2)
        b = off
        off += co
        off = (off + 7) & ~7
        convs.append((c1 + c2, co, w, b))
    lay["convs"] = convs
    lay["w_out"] = off
    off += 16
    lay["b_out"] = off
    off += 8
    lay["n"] = off
    return lay


def bf(x, emulate=True):
    return x.to(torch.bfloat16).to(x.dtype) if emulate else x


def unpack(params, emulate=True):
    p = torch.as_tensor(params, dtype=torch.float64)
    lay = layout()
    assert p.numel() == lay["n"], (p.numel(), lay["n"])
    w1 = p[lay["w_first"]:lay["w_first"] + 432].reshape(16, 1, 3, 3, 3)
    b1 = p[lay["b_first"]:lay["b_first"] + 16]
    convs = []
    for cin, co, w, b in lay["convs"]:
        W = p[w:w + co * 27 * cin].reshape(co, 27, cin).permute(0, 2, 1).reshape(co, cin, 3, 3, 3)
        convs.append((bf(W, emulate), p[b:b + co]))
    wo = p[lay["w_out"]:lay["w_out"] + 16].reshape(1, 16, 1, 1, 1)
    bo = p[lay["b_out"]:lay["b_out"] + 1]
    return w1, b1, convs, wo, bo


def forward(x, params, emulate=True):
    """x: [D, H, W] float64 tensor (may require grad through params)."""
    w1, b1, convs, wo, bo = params if isinstance(params, tuple) else unpack(params, emulate)
    v = x.reshape(1, 1, *x.shape)

    def conv(t, i):
        W, b = convs[i]
        return bf(F.relu(F.conv3d(t, W, b, padding=1)), emulate)

    def pool(t):
        return bf(F.avg_pool3d(t, 2), emulate)

    def up(t):
        return F.interpolate(t, scale_factor=2, mode="nearest")

    a0 = bf(F.relu(F.conv3d(v, w1, b1, padding=1)), emulate)
    e1 = conv(a0, 0)
    e2 = conv(conv(pool(e1), 1), 2)
    e3 = conv(conv(pool(e2), 3), 4)
    b = conv(conv(pool(e3), 5), 6)
    d3 = conv(conv(torch.cat([up(b), e3], 1), 7), 8)
    d2 = conv(conv(torch.cat([up(d3), e2], 1), 9), 10)
    d1 = conv(conv(torch.cat([up(d2), e1], 1), 11), 12)
    y = v + F.conv3d(d1, wo, bo)
    return y[0, 0]
