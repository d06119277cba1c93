// kv_unet.cu -- learned warm start: a small 3D U-Net (4 levels, 16/32/64/128
// channels, 3x3x3 convolutions, BF16 weights and activations, FP32
// accumulation) that maps a shift-and-add volume to an MLEM initial estimate,
// with its own training step (backpropagation + Adam).  No reference
// counterpart.
//
// Network (channels-last BF16 activations, D x H x W voxels, W % 128 == 0 for
// the 16-voxel rows of the coarsest level):
//   a0 = relu(conv(x: 1 -> 16))      e1 = relu(conv(a0: 16 -> 16))
//   a2 = relu(conv(pool(e1) -> 32))  e2 = relu(conv(a2: 32 -> 32))
//   a4 = relu(conv(pool(e2) -> 64))  e3 = relu(conv(a4: 64 -> 64))
//   a6 = relu(conv(pool(e3) -> 128)) b  = relu(conv(a6: 128 -> 128))
//   a8 = relu(conv(up(b) ++ e3 -> 64))   d3 = relu(conv(a8 -> 64))
//   a10 = relu(conv(up(d3) ++ e2 -> 32)) d2 = relu(conv(a10 -> 32))
//   a12 = relu(conv(up(d2) ++ e1 -> 16)) d1 = relu(conv(a12 -> 16))
//   y = x + conv1x1(d1: 16 -> 1)     (FP32 output)
// pool = 2x2x2 average, up = nearest x2, ++ = channel concatenation (read in
// place by the convolution, never copied).
#include "kv_conv_tc.cuh"
#include "kv_internal.h"
#include "kv_unet_kernels.cuh"

#include <cmath>
#include <cstring>
#include <random>

using unet::bf16;

namespace {

// ---------------------------------------------------------------- kernels

__global__ void conv_first_fwd(const float *__restrict__ x, const float *__restrict__ w /*[16][27]*/,
                               const float *__restrict__ b, bf16 *__restrict__ out, int D, int H, int W) {
    const long long n = (long long)D * H * W;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int xx = (int)(v % W);
        const long long zy = v / W;
        const int y = (int)(zy % H), z = (int)(zy / H);
        float in[27];
#pragma unroll
        for (int tap = 0; tap < 27; ++tap) {
            const int zz = z + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, x2 = xx + tap % 3 - 1;
            const bool ok = (unsigned)zz < (unsigned)D && (unsigned)yy < (unsigned)H && (unsigned)x2 < (unsigned)W;
            in[tap] = ok ? __ldg(x + ((long long)zz * H + yy) * W + x2) : 0.f;
        }
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
            float s0 = b[c], s1 = b[c + 1];
#pragma unroll
            for (int tap = 0; tap < 27; ++tap) {
                s0 = fmaf(w[c * 27 + tap], in[tap], s0);
                s1 = fmaf(w[(c + 1) * 27 + tap], in[tap], s1);
            }
            *reinterpret_cast<__nv_bfloat162 *>(out + v * 16 + c) = __floats2bfloat162_rn(fmaxf(s0, 0.f), fmaxf(s1, 0.f));
        }
    }
}

// dW0[c][tap] += sum_v dpre[v][c] * x[v + tap]  (blockIdx.y = tap), and the
// bias gradient when tap == 13 (the centre: every voxel contributes).
__global__ void conv_first_wgrad(const float *__restrict__ x, const bf16 *__restrict__ dpre, float *__restrict__ dw,
                                 float *__restrict__ db, int D, int H, int W) {
    const int tap = blockIdx.y;
    const long long n = (long long)D * H * W;
    float acc[16], accb[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = accb[c] = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int xx = (int)(v % W);
        const long long zy = v / W;
        const int y = (int)(zy % H), z = (int)(zy / H);
        const int zz = z + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, x2 = xx + tap % 3 - 1;
        const bool ok = (unsigned)zz < (unsigned)D && (unsigned)yy < (unsigned)H && (unsigned)x2 < (unsigned)W;
        const float xv = ok ? __ldg(x + ((long long)zz * H + yy) * W + x2) : 0.f;
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
            const float2 g = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(dpre + v * 16 + c));
            acc[c] = fmaf(g.x, xv, acc[c]);
            acc[c + 1] = fmaf(g.y, xv, acc[c + 1]);
            accb[c] += g.x;
            accb[c + 1] += g.y;
        }
    }
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        float s = acc[c], sb = accb[c];
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            sb += __shfl_xor_sync(0xffffffffu, sb, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(dw + c * 27 + tap, s);
            if (tap == 13) atomicAdd(db + c, sb);
        }
    }
}

// y[v] = x[v] + b + sum_c w[c] h[v][c]
__global__ void conv_out_fwd(const bf16 *__restrict__ h, const float *__restrict__ x, const float *__restrict__ w,
                             const float *__restrict__ b, float *__restrict__ y, long long n) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        float s = b[0];
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
            const float2 hv = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(h + v * 16 + c));
            s = fmaf(w[c], hv.x, s);
            s = fmaf(w[c + 1], hv.y, s);
        }
        y[v] = x[v] + s;
    }
}

// loss partials: sum (y - t)^2 per block; dy = 2 (y - t) / n.  A NaN target
// marks a voxel without a target: it adds nothing to the loss or gradient.
__global__ void mse_loss(const float *__restrict__ y, const float *__restrict__ t, float *__restrict__ dy, long long n,
                         double *__restrict__ partials) {
    double s = 0.0;
    const float scale = 2.f / (float)n;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float tv = t[v];
        if (tv != tv) {
            dy[v] = 0.f;
            continue;
        }
        const float d = y[v] - tv;
        s += (double)d * (double)d;
        dy[v] = scale * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) tot += sh[i];
        partials[blockIdx.x] = tot;
    }
}

__global__ void sum_loss(const double *__restrict__ partials, int nb, long long n, float *__restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < nb; ++i) s += partials[i];
        out[0] = (float)(s / (double)n);
    }
}

// backward of the output layer: dh[v][c] = w[c] dy[v]; dw[c] += sum dy h; db += sum dy
__global__ void conv_out_bwd(const bf16 *__restrict__ h, const float *__restrict__ dy, const float *__restrict__ w,
                             bf16 *__restrict__ dh, float *__restrict__ dw, float *__restrict__ db, long long n) {
    float acc[16], accb = 0.f;
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float g = dy[v];
        accb += g;
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
            const float2 hv = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(h + v * 16 + c));
            acc[c] = fmaf(g, hv.x, acc[c]);
            acc[c + 1] = fmaf(g, hv.y, acc[c + 1]);
            *reinterpret_cast<__nv_bfloat162 *>(dh + v * 16 + c) = __floats2bfloat162_rn(w[c] * g, w[c + 1] * g);
        }
    }
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        float s = acc[c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(dw + c, s);
    }
    for (int o = 16; o > 0; o >>= 1) accb += __shfl_xor_sync(0xffffffffu, accb, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(db, accb);
}

// 2x2x2 average pool (channels-last), out dims D/2 x H/2 x W/2
__global__ void avgpool_fwd(const bf16 *__restrict__ in, bf16 *__restrict__ out, int D, int H, int W, int C) {
    const int d2 = D / 2, h2 = H / 2, w2 = W / 2;
    const long long n = (long long)d2 * h2 * w2 * (C / 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % (C / 2)) * 2;
        const long long v = e / (C / 2);
        const int x = (int)(v % w2);
        const long long zy = v / w2;
        const int y = (int)(zy % h2), z = (int)(zy / h2);
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long src = ((long long)(2 * z + (k >> 2)) * H + (2 * y + ((k >> 1) & 1))) * W + 2 * x + (k & 1);
            const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(in + src * C + c));
            s0 += f.x;
            s1 += f.y;
        }
        *reinterpret_cast<__nv_bfloat162 *>(out + v * C + c) = __floats2bfloat162_rn(0.125f * s0, 0.125f * s1);
    }
}

// de[v][c] = (relu mask) * (dp[parent(v)][c] / 8 + dcat[v][c_off + c]) -- the gradient of an encoder output
// e = relu(...) from its pool and its skip connection, already masked by e > 0
__global__ void pool_bwd_skip_mask(const bf16 *__restrict__ dp, const bf16 *__restrict__ dcat, int ccat, int c_off,
                                   const bf16 *__restrict__ e, bf16 *__restrict__ de, int D, int H, int W, int C) {
    const long long n = (long long)D * H * W * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long v = i / C;
        const int x = (int)(v % W);
        const long long zy = v / W;
        const int y = (int)(zy % H), z = (int)(zy / H);
        const long long pv = ((long long)(z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
        float g = 0.125f * __bfloat162float(dp[pv * C + c]) + __bfloat162float(dcat[v * ccat + c_off + c]);
        if (!(__bfloat162float(e[i]) > 0.f)) g = 0.f;
        de[i] = __float2bfloat16_rn(g);
    }
}

// nearest x2 upsampling (channels-last): out D x H x W from in D/2 x H/2 x W/2
__global__ void upsample_fwd(const bf16 *__restrict__ in, bf16 *__restrict__ out, int D, int H, int W, int C) {
    const long long n = (long long)D * H * W * (C / 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % (C / 2)) * 2;
        const long long v = e / (C / 2);
        const int x = (int)(v % W);
        const long long zy = v / W;
        const int y = (int)(zy % H), z = (int)(zy / H);
        const long long pv = ((long long)(z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
        *reinterpret_cast<__nv_bfloat162 *>(out + v * C + c) = *reinterpret_cast<const __nv_bfloat162 *>(in + pv * C + c);
    }
}

// gradient through up(): dlow[p][c] = sum of the 8 children dcat[child][c] (channels [0,C) of a
// tensor with ccat channels), then masked by the relu output `a` of the low level
__global__ void upsample_bwd_mask(const bf16 *__restrict__ dcat, int ccat, const bf16 *__restrict__ a,
                                  bf16 *__restrict__ dlow, int D, int H, int W, int C) {
    // D, H, W: the low (half) resolution
    const long long n = (long long)D * H * W * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long v = i / C;
        const int x = (int)(v % W);
        const long long zy = v / W;
        const int y = (int)(zy % H), z = (int)(zy / H);
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long ch = ((long long)(2 * z + (k >> 2)) * (2 * H) + (2 * y + ((k >> 1) & 1))) * (2 * W) + 2 * x + (k & 1);
            s += __bfloat162float(dcat[ch * ccat + c]);
        }
        if (!(__bfloat162float(a[i]) > 0.f)) s = 0.f;
        dlow[i] = __float2bfloat16_rn(s);
    }
}

// g *= (a > 0), in place
__global__ void relu_mask(bf16 *__restrict__ g, const bf16 *__restrict__ a, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(a[i]) > 0.f)) g[i] = __float2bfloat16_rn(0.f);
}

// db[c] += sum_v g[v][c]
__global__ void bias_grad(const bf16 *__restrict__ g, float *__restrict__ db, long long nvox, int C) {
    extern __shared__ float sb[];
    for (int c = threadIdx.x; c < C; c += blockDim.x) sb[c] = 0.f;
    __syncthreads();
    const long long n = nvox * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        atomicAdd(&sb[i % C], __bfloat162float(g[i]));
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(db + c, sb[c]);
}

// Wt[ci][26 - tap][co] = W[co][tap][ci]: backward-data weights
__global__ void flip_transpose(const bf16 *__restrict__ w, bf16 *__restrict__ wt, int cout, int cin) {
    const int n = cout * 27 * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ci = i % cin, tap = (i / cin) % 27, co = i / (27 * cin);
        wt[((size_t)ci * 27 + (26 - tap)) * cout + co] = w[i];
    }
}

// Adam on the FP32 master parameters; refreshes the BF16 copies
__global__ void adam_step(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, bf16 *__restrict__ pb, size_t n, float lr, float b1, float b2,
                          float eps, const float *__restrict__ corr /* 1 - b1^t, 1 - b2^t */) {
    const float c1 = corr[0], c2 = corr[1];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16_rn(pi);
    }
}

__global__ void to_bf16(const float *__restrict__ in, bf16 *__restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

}  // namespace

// ------------------------------------------------------------------ model

struct kv_unet {
    kv_ctx *ctx = nullptr;
    // parameter layout
    struct Conv {
        int c1, c2, cout;
        size_t w, b;   // offsets into the flat parameter buffer
    };
    Conv conv[14];
    size_t w_first = 0, b_first = 0, w_out = 0, b_out = 0, nparams = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;   // FP32 master, grads, Adam moments
    bf16 *pb = nullptr;                                             // BF16 copy of the parameters
    bf16 *wt = nullptr;                                             // flipped / transposed weights
    long long step = 0;
    // activation workspace for one shape
    int D = 0, H = 0, W = 0;
    bool with_grads = false;
    std::vector<void *> bufs;
    bf16 *act[24] = {};
    bf16 *grad[24] = {};
    float *x = nullptr, *t = nullptr, *y = nullptr, *dy = nullptr, *loss = nullptr;
    double *partials = nullptr;
    float *corr = nullptr;                                          // Adam bias corrections (device)
    int *tc_status = nullptr;                                       // tensor-core convolution wait status
    cudaGraphExec_t train_graph = nullptr;
    float graph_lr = 0.f;
};

namespace {

enum {
    A0, E1, P1, A2, E2, P2, A4, E3, P3, A6, B, U3, A8, D3, U2, A10, D2, U1, A12, D1, CAT3, CAT2, CAT1, NACT
};

int grid_n(kv_ctx *ctx, long long n, int block = 256) {
    long long g = (n + block - 1) / block, cap = (long long)ctx->sm_count * 16;
    return (int)(g < cap ? (g < 1 ? 1 : g) : cap);
}

void free_workspace(kv_unet *u) {
    if (u->train_graph) cudaGraphExecDestroy(u->train_graph);
    u->train_graph = nullptr;
    for (void *b : u->bufs) cudaFree(b);
    u->bufs.clear();
    for (int i = 0; i < 24; ++i) u->act[i] = u->grad[i] = nullptr;
    u->x = u->t = u->y = u->dy = u->loss = nullptr;
    u->partials = nullptr;
    u->D = u->H = u->W = 0;
}

kv_status alloc(kv_unet *u, void **p, size_t bytes) {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return kv_fail(u->ctx, KV_ERR_OOM, "U-Net workspace (%zu bytes)", bytes);
    }
    u->bufs.push_back(*p);
    return KV_OK;
}

// channel count and resolution level (0 = full) of each activation
void act_shape(int i, int &c, int &lvl) {
    static const int C[NACT] = {16, 16, 16, 32, 32, 32, 64, 64, 64, 128, 128, 128, 64, 64, 64, 32, 32, 32, 16, 16, 192, 96, 48};
    static const int L[NACT] = {0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 2, 2, 1, 1, 1, 0, 0, 0, 2, 1, 0};
    c = C[i];
    lvl = L[i];
}

kv_status ensure_workspace(kv_unet *u, int D, int H, int W, bool grads) {
    if (u->D == D && u->H == H && u->W == W && (u->with_grads || !grads)) return KV_OK;
    free_workspace(u);
    if (D % 8 || H % 8 || W % 128)
        return kv_fail(u->ctx, KV_ERR_INVALID_ARG, "U-Net input must be D, H multiples of 8 and W of 128 (got %d x %d x %d)",
                       D, H, W);
    const long long n0 = (long long)D * H * W;
    for (int i = 0; i < NACT; ++i) {
        int c, l;
        act_shape(i, c, l);
        const long long nv = n0 >> (3 * l);
        if (i >= CAT3 && !grads) continue;   // concatenation gradients: training only
        KV_TRY(alloc(u, (void **)&u->act[i], (size_t)nv * c * sizeof(bf16)));
        if (grads) KV_TRY(alloc(u, (void **)&u->grad[i], (size_t)nv * c * sizeof(bf16)));
    }
    KV_TRY(alloc(u, (void **)&u->x, n0 * sizeof(float)));
    KV_TRY(alloc(u, (void **)&u->y, n0 * sizeof(float)));
    if (grads) {
        KV_TRY(alloc(u, (void **)&u->t, n0 * sizeof(float)));
        KV_TRY(alloc(u, (void **)&u->dy, n0 * sizeof(float)));
        KV_TRY(alloc(u, (void **)&u->loss, sizeof(float) * 4));
        KV_TRY(alloc(u, (void **)&u->partials, sizeof(double) * 4096));
    }
    u->D = D;
    u->H = H;
    u->W = W;
    u->with_grads = grads;
    return KV_OK;
}

// forward convolution over all output channels (chunks of <= 64)
kv_status conv3(kv_unet *u, int layer, const bf16 *in1, const bf16 *in2, bf16 *out, int lvl, bool weights_t,
                int c_in_override = -1) {
    const kv_unet::Conv &L = u->conv[layer];
    kv_ctx *ctx = u->ctx;
    const int D = u->D >> lvl, H = u->H >> lvl, W = u->W >> lvl;
    const long long nvox = (long long)D * H * W;
    // forward: in1 (c1) ++ in2 (c2) -> cout with W; backward-data: in1 = dPre (cout) -> c1 + c2 with Wt
    const int c1 = weights_t ? L.cout : L.c1, c2 = weights_t ? 0 : L.c2;
    const int cout = weights_t ? (c_in_override > 0 ? c_in_override : L.c1 + L.c2) : L.cout;
    const bf16 *w = weights_t ? u->wt + L.w : u->pb + L.w;
    const float *bias = weights_t ? nullptr : u->p + L.b;
    const int blocks = (int)((nvox / 16 + 3) / 4);
    LaunchTimer lt(ctx, weights_t ? "unet_conv_dgrad" : "unet_conv_fwd");
    int bw, bh, bd;
    if (convtc::tile_shape(D, H, W, bw, bh, bd)) {
        // tcgen05 / TMA implicit GEMM (kv_conv_tc.cuh)
        const char *why = convtc::launch(in1, c1, in2, c2, w, bias, !weights_t, out, cout, D, H, W, u->tc_status,
                                         ctx->sm_count, ctx->stream);
        if (why != nullptr) return kv_fail(ctx, KV_ERR_UNSUPPORTED, "tensor-core convolution: %s", why);
        KV_CHECK_LAUNCH(ctx, "unet conv3 (tcgen05)");
        return KV_OK;
    }
    // volumes that are not a whole number of 128-voxel tiles (the deepest
    // levels of small inputs): warp-level mma.sync
    for (int n0 = 0; n0 < cout; n0 += 64) {
        const int nc = cout - n0 < 64 ? cout - n0 : 64;
        const bool relu = !weights_t;
        switch (nc) {
        case 16: relu ? unet::conv3_fwd<2, true><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W)
                      : unet::conv3_fwd<2, false><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W); break;
        case 32: relu ? unet::conv3_fwd<4, true><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W)
                      : unet::conv3_fwd<4, false><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W); break;
        case 48: relu ? unet::conv3_fwd<6, true><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W)
                      : unet::conv3_fwd<6, false><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W); break;
        case 64: relu ? unet::conv3_fwd<8, true><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W)
                      : unet::conv3_fwd<8, false><<<blocks, 128, 0, ctx->stream>>>(in1, c1, in2, c2, w, bias, out, cout, n0, D, H, W); break;
        default: return kv_fail(ctx, KV_ERR_UNSUPPORTED, "conv chunk of %d channels", nc);
        }
    }
    KV_CHECK_LAUNCH(ctx, "unet conv3");
    return KV_OK;
}

kv_status wgrad(kv_unet *u, int layer, const bf16 *dpre, const bf16 *in1, const bf16 *in2, int lvl) {
    const kv_unet::Conv &L = u->conv[layer];
    kv_ctx *ctx = u->ctx;
    const int D = u->D >> lvl, H = u->H >> lvl, W = u->W >> lvl;
    const long long nvox = (long long)D * H * W;
    const int cin = L.c1 + L.c2;
    const int ntw = cin % 64 == 0 ? 8 : (cin % 32 == 0 ? 4 : 2);
    const int groups = cin / (8 * ntw);
    long long chunk = 16384;
    while (chunk > 1024 && (nvox + chunk - 1) / chunk < ctx->sm_count / 4) chunk /= 2;
    dim3 grid((unsigned)((nvox + chunk - 1) / chunk), 27, (L.cout / 16) * groups);
    float *dw = u->g + L.w;
    LaunchTimer lt(ctx, "unet_conv_wgrad");
    switch (ntw) {
    case 8: unet::conv3_wgrad<8><<<grid, 128, 0, ctx->stream>>>(dpre, L.cout, in1, L.c1, in2, L.c2, dw, D, H, W, (int)chunk); break;
    case 4: unet::conv3_wgrad<4><<<grid, 128, 0, ctx->stream>>>(dpre, L.cout, in1, L.c1, in2, L.c2, dw, D, H, W, (int)chunk); break;
    default: unet::conv3_wgrad<2><<<grid, 128, 0, ctx->stream>>>(dpre, L.cout, in1, L.c1, in2, L.c2, dw, D, H, W, (int)chunk); break;
    }
    {
        LaunchTimer lb(ctx, "unet_bias_grad");
        bias_grad<<<grid_n(ctx, nvox * L.cout), 256, L.cout * sizeof(float), ctx->stream>>>(dpre, u->g + L.b, nvox, L.cout);
    }
    KV_CHECK_LAUNCH(ctx, "unet wgrad");
    return KV_OK;
}

kv_status forward(kv_unet *u) {
    kv_ctx *ctx = u->ctx;
    const int D = u->D, H = u->H, W = u->W;
    const long long n0 = (long long)D * H * W;
    bf16 **a = u->act;
    {
        LaunchTimer lt(ctx, "unet_conv_first");
        conv_first_fwd<<<grid_n(ctx, n0), 256, 0, ctx->stream>>>(u->x, u->p + u->w_first, u->p + u->b_first, a[A0], D, H, W);
    }
    KV_TRY(conv3(u, 0, a[A0], nullptr, a[E1], 0, false));
    avgpool_fwd<<<grid_n(ctx, (n0 >> 3) * 8), 256, 0, ctx->stream>>>(a[E1], a[P1], D, H, W, 16);
    KV_TRY(conv3(u, 1, a[P1], nullptr, a[A2], 1, false));
    KV_TRY(conv3(u, 2, a[A2], nullptr, a[E2], 1, false));
    avgpool_fwd<<<grid_n(ctx, (n0 >> 6) * 16), 256, 0, ctx->stream>>>(a[E2], a[P2], D >> 1, H >> 1, W >> 1, 32);
    KV_TRY(conv3(u, 3, a[P2], nullptr, a[A4], 2, false));
    KV_TRY(conv3(u, 4, a[A4], nullptr, a[E3], 2, false));
    avgpool_fwd<<<grid_n(ctx, (n0 >> 9) * 32), 256, 0, ctx->stream>>>(a[E3], a[P3], D >> 2, H >> 2, W >> 2, 64);
    KV_TRY(conv3(u, 5, a[P3], nullptr, a[A6], 3, false));
    KV_TRY(conv3(u, 6, a[A6], nullptr, a[B], 3, false));
    upsample_fwd<<<grid_n(ctx, (n0 >> 6) * 64), 256, 0, ctx->stream>>>(a[B], a[U3], D >> 2, H >> 2, W >> 2, 128);
    KV_TRY(conv3(u, 7, a[U3], a[E3], a[A8], 2, false));
    KV_TRY(conv3(u, 8, a[A8], nullptr, a[D3], 2, false));
    upsample_fwd<<<grid_n(ctx, (n0 >> 3) * 32), 256, 0, ctx->stream>>>(a[D3], a[U2], D >> 1, H >> 1, W >> 1, 64);
    KV_TRY(conv3(u, 9, a[U2], a[E2], a[A10], 1, false));
    KV_TRY(conv3(u, 10, a[A10], nullptr, a[D2], 1, false));
    upsample_fwd<<<grid_n(ctx, n0 * 16), 256, 0, ctx->stream>>>(a[D2], a[U1], D, H, W, 32);
    KV_TRY(conv3(u, 11, a[U1], a[E1], a[A12], 0, false));
    KV_TRY(conv3(u, 12, a[A12], nullptr, a[D1], 0, false));
    {
        LaunchTimer lt(ctx, "unet_conv_out");
        conv_out_fwd<<<grid_n(ctx, n0), 256, 0, ctx->stream>>>(a[D1], u->x, u->p + u->w_out, u->p + u->b_out, u->y, n0);
    }
    KV_CHECK_LAUNCH(ctx, "unet forward");
    return KV_OK;
}

// backward of a conv + relu layer whose output gradient (already masked by
// the layer's relu) is dpre: weight / bias gradients and the input gradient
// into dx (unmasked; c_dx channels)
kv_status conv_backward(kv_unet *u, int layer, const bf16 *dpre, const bf16 *in1, const bf16 *in2, bf16 *dx, int lvl) {
    KV_TRY(wgrad(u, layer, dpre, in1, in2, lvl));
    if (dx != nullptr) KV_TRY(conv3(u, layer, dpre, nullptr, dx, lvl, true));
    return KV_OK;
}

kv_status backward(kv_unet *u) {
    kv_ctx *ctx = u->ctx;
    const int D = u->D, H = u->H, W = u->W;
    const long long n0 = (long long)D * H * W;
    bf16 **a = u->act, **g = u->grad;
    // weights for the backward-data convolutions
    for (int l = 0; l < 14; ++l) {
        const kv_unet::Conv &L = u->conv[l];
        if (L.cout == 0) continue;
        const int n = L.cout * 27 * (L.c1 + L.c2);
        flip_transpose<<<(n + 255) / 256, 256, 0, ctx->stream>>>(u->pb + L.w, u->wt + L.w, L.cout, L.c1 + L.c2);
    }
    // output layer
    conv_out_bwd<<<grid_n(ctx, n0), 256, 0, ctx->stream>>>(a[D1], u->dy, u->p + u->w_out, g[D1], u->g + u->w_out,
                                                           u->g + u->b_out, n0);
    relu_mask<<<grid_n(ctx, n0 * 16), 256, 0, ctx->stream>>>(g[D1], a[D1], n0 * 16);
    // level 0 decoder
    KV_TRY(conv_backward(u, 12, g[D1], a[A12], nullptr, g[A12], 0));
    relu_mask<<<grid_n(ctx, n0 * 16), 256, 0, ctx->stream>>>(g[A12], a[A12], n0 * 16);
    KV_TRY(conv_backward(u, 11, g[A12], a[U1], a[E1], g[CAT1], 0));      // 48 ch: up(d2) 32 ++ e1 16
    upsample_bwd_mask<<<grid_n(ctx, (n0 >> 3) * 32), 256, 0, ctx->stream>>>(g[CAT1], 48, a[D2], g[D2], D >> 1, H >> 1, W >> 1, 32);
    // level 1 decoder
    KV_TRY(conv_backward(u, 10, g[D2], a[A10], nullptr, g[A10], 1));
    relu_mask<<<grid_n(ctx, (n0 >> 3) * 32), 256, 0, ctx->stream>>>(g[A10], a[A10], (n0 >> 3) * 32);
    KV_TRY(conv_backward(u, 9, g[A10], a[U2], a[E2], g[CAT2], 1));       // 96 ch: up(d3) 64 ++ e2 32
    upsample_bwd_mask<<<grid_n(ctx, (n0 >> 6) * 64), 256, 0, ctx->stream>>>(g[CAT2], 96, a[D3], g[D3], D >> 2, H >> 2, W >> 2, 64);
    // level 2 decoder
    KV_TRY(conv_backward(u, 8, g[D3], a[A8], nullptr, g[A8], 2));
    relu_mask<<<grid_n(ctx, (n0 >> 6) * 64), 256, 0, ctx->stream>>>(g[A8], a[A8], (n0 >> 6) * 64);
    KV_TRY(conv_backward(u, 7, g[A8], a[U3], a[E3], g[CAT3], 2));        // 192 ch: up(b) 128 ++ e3 64
    upsample_bwd_mask<<<grid_n(ctx, (n0 >> 9) * 128), 256, 0, ctx->stream>>>(g[CAT3], 192, a[B], g[B], D >> 3, H >> 3, W >> 3, 128);
    // bottleneck
    KV_TRY(conv_backward(u, 6, g[B], a[A6], nullptr, g[A6], 3));
    relu_mask<<<grid_n(ctx, (n0 >> 9) * 128), 256, 0, ctx->stream>>>(g[A6], a[A6], (n0 >> 9) * 128);
    KV_TRY(conv_backward(u, 5, g[A6], a[P3], nullptr, g[P3], 3));
    pool_bwd_skip_mask<<<grid_n(ctx, (n0 >> 6) * 64), 256, 0, ctx->stream>>>(g[P3], g[CAT3], 192, 128, a[E3], g[E3],
                                                                             D >> 2, H >> 2, W >> 2, 64);
    // level 2 encoder
    KV_TRY(conv_backward(u, 4, g[E3], a[A4], nullptr, g[A4], 2));
    relu_mask<<<grid_n(ctx, (n0 >> 6) * 64), 256, 0, ctx->stream>>>(g[A4], a[A4], (n0 >> 6) * 64);
    KV_TRY(conv_backward(u, 3, g[A4], a[P2], nullptr, g[P2], 2));
    pool_bwd_skip_mask<<<grid_n(ctx, (n0 >> 3) * 32), 256, 0, ctx->stream>>>(g[P2], g[CAT2], 96, 64, a[E2], g[E2],
                                                                             D >> 1, H >> 1, W >> 1, 32);
    // level 1 encoder
    KV_TRY(conv_backward(u, 2, g[E2], a[A2], nullptr, g[A2], 1));
    relu_mask<<<grid_n(ctx, (n0 >> 3) * 32), 256, 0, ctx->stream>>>(g[A2], a[A2], (n0 >> 3) * 32);
    KV_TRY(conv_backward(u, 1, g[A2], a[P1], nullptr, g[P1], 1));
    pool_bwd_skip_mask<<<grid_n(ctx, n0 * 16), 256, 0, ctx->stream>>>(g[P1], g[CAT1], 48, 32, a[E1], g[E1], D, H, W, 16);
    // level 0 encoder
    KV_TRY(conv_backward(u, 0, g[E1], a[A0], nullptr, g[A0], 0));
    relu_mask<<<grid_n(ctx, n0 * 16), 256, 0, ctx->stream>>>(g[A0], a[A0], n0 * 16);
    {
        dim3 grid(grid_n(ctx, n0) > 1024 ? 1024 : grid_n(ctx, n0), 27);
        conv_first_wgrad<<<grid, 256, 0, ctx->stream>>>(u->x, g[A0], u->g + u->w_first, u->g + u->b_first, D, H, W);
    }
    KV_CHECK_LAUNCH(ctx, "unet backward");
    return KV_OK;
}

kv_status loss_and_grad(kv_unet *u) {
    kv_ctx *ctx = u->ctx;
    const long long n0 = (long long)u->D * u->H * u->W;
    const int nb = grid_n(ctx, n0) > 4096 ? 4096 : grid_n(ctx, n0);
    mse_loss<<<nb, 256, 0, ctx->stream>>>(u->y, u->t, u->dy, n0, u->partials);
    sum_loss<<<1, 32, 0, ctx->stream>>>(u->partials, nb, n0, u->loss);
    KV_CHECK_LAUNCH(ctx, "unet loss");
    return KV_OK;
}

kv_status train_body(kv_unet *u, float lr, bool apply) {
    kv_ctx *ctx = u->ctx;
    KV_TRY(forward(u));
    KV_TRY(loss_and_grad(u));
    KV_CHECK_CUDA(ctx, cudaMemsetAsync(u->g, 0, u->nparams * sizeof(float), ctx->stream));
    KV_TRY(backward(u));
    if (apply) {
        adam_step<<<grid_n(ctx, (long long)u->nparams), 256, 0, ctx->stream>>>(u->p, u->g, u->m, u->v, u->pb, u->nparams, lr,
                                                                             0.9f, 0.999f, 1e-8f, u->corr);
        KV_CHECK_LAUNCH(ctx, "adam");
    }
    return KV_OK;
}

kv_status copy_in(kv_unet *u, float *dst, const float *src, size_t n, kv_mem mem) {
    KV_CHECK_CUDA(u->ctx, cudaMemcpyAsync(dst, src, n * sizeof(float),
                                          mem == KV_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                          u->ctx->stream));
    return KV_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" kv_status kv_unet_create(kv_ctx *ctx, uint64_t seed, kv_unet **out) {
    if (ctx == nullptr || out == nullptr) return KV_ERR_INVALID_ARG;
    *out = nullptr;
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    kv_unet *u = new (std::nothrow) kv_unet;
    if (u == nullptr) return KV_ERR_OOM;
    u->ctx = ctx;
    ctx->plans += 1;   // the network keeps the context alive like a plan
    const int spec[14][3] = {{16, 0, 16},  {16, 0, 32},   {32, 0, 32},  {32, 0, 64},  {64, 0, 64},
                             {64, 0, 128}, {128, 0, 128}, {128, 64, 64}, {64, 0, 64}, {64, 32, 32},
                             {32, 0, 32},  {32, 16, 16},  {16, 0, 16},   {0, 0, 0}};
    size_t off = 0;
    u->w_first = off;
    off += 16 * 27;
    u->b_first = off;
    off += 16;
    for (int l = 0; l < 14; ++l) {
        u->conv[l] = {spec[l][0], spec[l][1], spec[l][2], 0, 0};
        if (spec[l][2] == 0) continue;
        u->conv[l].w = off;
        off += (size_t)spec[l][2] * 27 * (spec[l][0] + spec[l][1]);
        u->conv[l].b = off;
        off += spec[l][2];
        off = (off + 7) & ~(size_t)7;   // keep every weight block 16-byte aligned in BF16
    }
    u->w_out = off;
    off += 16;
    u->b_out = off;
    off += 8;
    u->nparams = off;
    // He initialisation (normal, std sqrt(2 / fan_in)); zero biases; the output
    // layer starts at zero so the untrained network returns its input
    std::vector<float> h(off, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](size_t o, size_t n, int fan_in) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)fan_in));
        for (size_t i = 0; i < n; ++i) h[o + i] = nd(rng);
    };
    fill(u->w_first, 16 * 27, 27);
    for (int l = 0; l < 13; ++l) {
        const auto &L = u->conv[l];
        fill(L.w, (size_t)L.cout * 27 * (L.c1 + L.c2), 27 * (L.c1 + L.c2));
    }
    kv_status s = KV_OK;
    if (cudaMalloc((void **)&u->p, off * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&u->g, off * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&u->m, off * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&u->v, off * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&u->pb, off * sizeof(bf16)) != cudaSuccess ||
        cudaMalloc((void **)&u->wt, off * sizeof(bf16)) != cudaSuccess ||
        cudaMalloc((void **)&u->corr, 4 * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&u->tc_status, sizeof(int)) != cudaSuccess) {
        s = kv_fail(ctx, KV_ERR_OOM, "U-Net parameters");
    } else {
        cudaMemcpy(u->p, h.data(), off * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemset(u->m, 0, off * sizeof(float));
        cudaMemset(u->v, 0, off * sizeof(float));
        cudaMemset(u->tc_status, 0, sizeof(int));
        to_bf16<<<grid_n(ctx, (long long)off), 256, 0, ctx->stream>>>(u->p, u->pb, off);
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) s = kv_fail(ctx, KV_ERR_CUDA, "U-Net init");
    }
    if (s != KV_OK) {
        kv_unet_destroy(u);
        return s;
    }
    *out = u;
    return KV_OK;
}

extern "C" kv_status kv_unet_destroy(kv_unet *u) {
    if (u == nullptr) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = u->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    free_workspace(u);
    cudaFree(u->p);
    cudaFree(u->g);
    cudaFree(u->m);
    cudaFree(u->v);
    cudaFree(u->pb);
    cudaFree(u->wt);
    cudaFree(u->corr);
    cudaFree(u->tc_status);
    delete u;
    kv_ctx_release_ref(ctx);
    return KV_OK;
}

extern "C" size_t kv_unet_num_params(const kv_unet *u) { return u ? u->nparams : 0; }

namespace {
// Reads (and clears) the tensor-core convolution's wait status: non-zero when
// one of its bounded pipeline waits gave up.  Synchronises the stream.
kv_status tc_check(kv_unet *u) {
    kv_ctx *ctx = u->ctx;
    int h = 0;
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(&h, u->tc_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h != 0) {
        cudaMemset(u->tc_status, 0, sizeof(int));
        return kv_fail(ctx, KV_ERR_TIMEOUT, "tensor-core convolution: pipeline wait %d timed out", h);
    }
    return KV_OK;
}
}  // namespace

extern "C" kv_status kv_unet_forward(kv_unet *u, const float *in, float *out, int32_t D, int32_t H, int32_t W,
                                     kv_mem mem) {
    if (u == nullptr || in == nullptr || out == nullptr) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = u->ctx;
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    KV_TRY(ensure_workspace(u, D, H, W, false));
    const size_t n = (size_t)D * H * W;
    KV_TRY(copy_in(u, u->x, in, n, mem));
    KV_TRY(forward(u));
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(out, u->y, n * sizeof(float),
                                       mem == KV_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, ctx->stream));
    return tc_check(u);
}

// One Adam step on (input, target); loss = mean squared error before the step.
// The step (forward, loss, backward, update) runs as a CUDA graph captured on
// the first call for a given shape and learning rate.
extern "C" kv_status kv_unet_train_step(kv_unet *u, const float *in, const float *target, int32_t D, int32_t H,
                                        int32_t W, float lr, float *loss, kv_mem mem) {
    if (u == nullptr || in == nullptr || target == nullptr) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = u->ctx;
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    KV_TRY(ensure_workspace(u, D, H, W, true));
    const size_t n = (size_t)D * H * W;
    KV_TRY(copy_in(u, u->x, in, n, mem));
    KV_TRY(copy_in(u, u->t, target, n, mem));
    // Adam bias corrections of this step go to device memory, so the captured
    // step stays valid from one step to the next
    const float corr[2] = {1.f - powf(0.9f, (float)(u->step + 1)), 1.f - powf(0.999f, (float)(u->step + 1))};
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(u->corr, corr, sizeof corr, cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->timing) {
        KV_TRY(train_body(u, lr, true));          // traced: plain launches
    } else {
        if (u->train_graph == nullptr || u->graph_lr != lr) {
            if (u->train_graph) {
                KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                cudaGraphExecDestroy(u->train_graph);
                u->train_graph = nullptr;
            }
            cudaStream_t user = ctx->stream;
            ctx->stream = ctx->own_stream;
            KV_CHECK_CUDA(ctx, cudaStreamBeginCapture(ctx->own_stream, cudaStreamCaptureModeThreadLocal));
            kv_status st = train_body(u, lr, true);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(ctx->own_stream, &graph);
            ctx->stream = user;
            if (st != KV_OK) {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            if (e != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "train step capture: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&u->train_graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                u->train_graph = nullptr;
                return kv_fail(ctx, KV_ERR_CUDA, "train step instantiate: %s", cudaGetErrorString(e));
            }
            u->graph_lr = lr;
        }
        KV_CHECK_CUDA(ctx, cudaGraphLaunch(u->train_graph, ctx->stream));
    }
    u->step += 1;
    if (loss) KV_CHECK_CUDA(ctx, cudaMemcpyAsync(loss, u->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    return tc_check(u);
}

// Loss and FP32 parameter gradients (no update), for gradient checks.
extern "C" kv_status kv_unet_gradients(kv_unet *u, const float *in, const float *target, int32_t D, int32_t H,
                                       int32_t W, float *loss, float *grads, kv_mem mem) {
    if (u == nullptr || in == nullptr || target == nullptr || grads == nullptr) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = u->ctx;
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    KV_TRY(ensure_workspace(u, D, H, W, true));
    const size_t n = (size_t)D * H * W;
    KV_TRY(copy_in(u, u->x, in, n, mem));
    KV_TRY(copy_in(u, u->t, target, n, mem));
    KV_TRY(train_body(u, 0.f, false));
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(grads, u->g, u->nparams * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (loss) KV_CHECK_CUDA(ctx, cudaMemcpyAsync(loss, u->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    return tc_check(u);
}

// State = parameters, Adam first and second moments (3 * num_params floats)
// and the step count, for checkpoints.
extern "C" kv_status kv_unet_get_state(const kv_unet *u, float *state, int64_t *step) {
    if (u == nullptr || state == nullptr) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = u->ctx;
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    KV_CHECK_CUDA(ctx, cudaMemcpy(state, u->p, u->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    KV_CHECK_CUDA(ctx, cudaMemcpy(state + u->nparams, u->m, u->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    KV_CHECK_CUDA(ctx, cudaMemcpy(state + 2 * u->nparams, u->v, u->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    if (step) *step = u->step;
    return KV_OK;
}

extern "C" kv_status kv_unet_set_state(kv_unet *u, const float *state, int64_t step) {
    if (u == nullptr || state == nullptr || step < 0) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = u->ctx;
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    KV_CHECK_CUDA(ctx, cudaMemcpy(u->p, state, u->nparams * sizeof(float), cudaMemcpyHostToDevice));
    KV_CHECK_CUDA(ctx, cudaMemcpy(u->m, state + u->nparams, u->nparams * sizeof(float), cudaMemcpyHostToDevice));
    KV_CHECK_CUDA(ctx, cudaMemcpy(u->v, state + 2 * u->nparams, u->nparams * sizeof(float), cudaMemcpyHostToDevice));
    to_bf16<<<grid_n(ctx, (long long)u->nparams), 256, 0, ctx->stream>>>(u->p, u->pb, u->nparams);
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    u->step = step;
    return KV_OK;
}

// One 3x3x3 convolution of the network's kind on caller buffers (device
// pointers, BF16 bit patterns): the operator behind every U-Net layer, for
// callers and tests that need a single layer.  kernel: 0 = the tensor-core
// (tcgen05 / TMA) kernel where the volume tiles, else mma.sync; 1 = tcgen05
// only; 2 = mma.sync only.
extern "C" kv_status kv_conv3_bf16(kv_ctx *ctx, const uint16_t *in1, int32_t c1, const uint16_t *in2, int32_t c2,
                                   const uint16_t *w, const float *bias, int32_t relu, uint16_t *out, int32_t cout,
                                   int32_t D, int32_t H, int32_t W, int32_t kernel) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (in1 == nullptr || w == nullptr || out == nullptr || (c2 > 0 && in2 == nullptr))
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_conv3_bf16: null buffer");
    if (D <= 0 || H <= 0 || W <= 0 || c1 <= 0 || c2 < 0 || cout <= 0 || kernel < 0 || kernel > 2)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_conv3_bf16: bad sizes or kernel choice");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    const bf16 *a = reinterpret_cast<const bf16 *>(in1), *b = reinterpret_cast<const bf16 *>(in2);
    const bf16 *wb = reinterpret_cast<const bf16 *>(w);
    bf16 *o = reinterpret_cast<bf16 *>(out);
    int bw, bh, bd;
    const bool tiles = convtc::tile_shape(D, H, W, bw, bh, bd);
    if (kernel == 1 && !tiles)
        return kv_fail(ctx, KV_ERR_UNSUPPORTED, "kv_conv3_bf16: the volume is not a whole number of 128-voxel tiles");
    if (kernel != 2 && tiles) {
        const char *why = convtc::launch(a, c1, c2 ? b : nullptr, c2, wb, bias, relu != 0, o, cout, D, H, W,
                                         ctx->d_status, ctx->sm_count, ctx->stream);
        if (why != nullptr) return kv_fail(ctx, KV_ERR_UNSUPPORTED, "tensor-core convolution: %s", why);
        KV_CHECK_LAUNCH(ctx, "kv_conv3_bf16 (tcgen05)");
        return KV_OK;
    }
    if (W % 16 != 0 || c1 % 16 != 0 || c2 % 16 != 0 || cout % 16 != 0)
        return kv_fail(ctx, KV_ERR_UNSUPPORTED, "kv_conv3_bf16: mma.sync needs W, channels multiples of 16");
    const long long nvox = (long long)D * H * W;
    const int blocks = (int)((nvox / 16 + 3) / 4);
    for (int n0 = 0; n0 < cout; n0 += 64) {
        const int nc = cout - n0 < 64 ? cout - n0 : 64;
        const bool rl = relu != 0;
        switch (nc) {
        case 16: rl ? unet::conv3_fwd<2, true><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W)
                    : unet::conv3_fwd<2, false><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W); break;
        case 32: rl ? unet::conv3_fwd<4, true><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W)
                    : unet::conv3_fwd<4, false><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W); break;
        case 48: rl ? unet::conv3_fwd<6, true><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W)
                    : unet::conv3_fwd<6, false><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W); break;
        default: rl ? unet::conv3_fwd<8, true><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W)
                    : unet::conv3_fwd<8, false><<<blocks, 128, 0, ctx->stream>>>(a, c1, b, c2, wb, bias, o, cout, n0, D, H, W); break;
        }
    }
    KV_CHECK_LAUNCH(ctx, "kv_conv3_bf16 (mma.sync)");
    return KV_OK;
}
