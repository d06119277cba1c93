// kv_misc.cu -- shift-and-add, phantom rasteriser and elementwise kernels.
#include "kv_internal.h"
#include "kv_tma.cuh"

#include <algorithm>
#include <cmath>

namespace {

// Shift-and-add (recons::ShiftAndAdd, Reconstructors.h:263-379):
// out[k][v][u] = (1/P) * sum_i in[i][v + t_ki][u], zero outside the ROI.
// The reference sums the weighted views in double (vtkImageWeightedSum); here
// the views are summed exactly enough with a float-float (TwoSum) accumulator
// and the mean is formed in double before rounding to float.
// Block: 32 columns x 8 rows; each thread loops over a batch of slices so that
// consecutive slices, whose shifts differ by a few rows, hit the same lines.
__global__ void __launch_bounds__(256) saa_kernel(int nu, int nv, int nz, int P,
                                                  const int32_t *__restrict__ shift,
                                                  const float *__restrict__ proj,
                                                  float *__restrict__ out, int kb) {
    extern __shared__ int32_t sh_shift[];
    const int u = blockIdx.x * 32 + threadIdx.x;
    const int v = blockIdx.y * blockDim.y + threadIdx.y;
    const int k0 = blockIdx.z * kb, k1 = min(nz, k0 + kb);
    for (int t = threadIdx.y * 32 + threadIdx.x; t < (k1 - k0) * P; t += blockDim.x * blockDim.y)
        sh_shift[t] = shift[(size_t)k0 * P + t];
    __syncthreads();
    if (u >= nu || v >= nv) return;
    const double w = 1.0 / (double)P;
    for (int k = k0; k < k1; ++k) {
        float hi = 0.f, lo = 0.f;
        const int32_t *sk = sh_shift + (size_t)(k - k0) * P;
        for (int i = 0; i < P; ++i) {
            const int r = v + sk[i];
            if (r >= 0 && r < nv) {
                const float x = __ldg(proj + ((size_t)i * nv + r) * nu + u);
                const float s = hi + x;                       // TwoSum(hi, x)
                const float bp = s - hi;
                const float err = (hi - (s - bp)) + (x - bp);
                hi = s;
                lo += err;
            }
        }
        out[((size_t)k * nv + v) * nu + u] = (float)(((double)hi + (double)lo) * w);
    }
}

// The same sums with each view's rows staged in shared memory.  A block
// covers 32 detector columns x kSaaRows rows x kSaaSlices slices; for every
// view one thread loads, by TMA, the band of that view's rows the block's
// shifted rows reach (kSaaRows + the largest spread of the block's shifts;
// rows outside the detector read zeros, which is the reference's zero
// padding) into a ring of shared-memory stages, and every thread adds its
// kSaaRows / 8 x kSaaSlices outputs' rows from the band.  Views are added in
// the same order with the same TwoSum as saa_kernel, and a row outside the
// detector adds an exact zero, so the two kernels agree bit for bit.
constexpr int kSaaRows = 32, kSaaSlices = 4, kSaaStages = 3;
constexpr uint32_t kSaaWaitPolls = 1u << 22;

__global__ void __launch_bounds__(256) saa_band_kernel(const __grid_constant__ CUtensorMap pmap, int nu, int nv,
                                                       int nz, int P, const int32_t *__restrict__ shift,
                                                       float *__restrict__ out, int nb, uint32_t stage_stride,
                                                       int *status) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[kSaaStages];
    __shared__ int bstart[kSaaStages];
    unsigned char *base = smem + ((128u - (kvtma::smem_u32(smem) & 127u)) & 127u);
    float *bands = reinterpret_cast<float *>(base);
    int *sh = reinterpret_cast<int *>(base + kSaaStages * stage_stride);     // [kSaaSlices][P]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int u0 = blockIdx.x * 32, v0 = blockIdx.y * kSaaRows, k0 = blockIdx.z * kSaaSlices;
    const int kn = min(kSaaSlices, nz - k0);
    for (int t = threadIdx.x; t < kn * P; t += blockDim.x) sh[t] = shift[(size_t)k0 * P + t];
    if (threadIdx.x == 0) {
        for (int s = 0; s < kSaaStages; ++s) kvtma::mbar_init(&full[s], 1);
        kvtma::fence_mbar_init();
    }
    __syncthreads();
    const uint32_t band_bytes = 32u * (uint32_t)nb * 4u;
    auto issue = [&](int i, int st) {
        int tmin = sh[i];
        for (int kk = 1; kk < kn; ++kk) tmin = min(tmin, sh[kk * P + i]);
        const int bs = v0 + tmin;
        bstart[st] = bs;
        kvtma::fence_proxy_async_smem();
        kvtma::mbar_arrive_expect_tx(&full[st], band_bytes);
        kvtma::tma_load_3d(kvtma::smem_u32(base + (size_t)st * stage_stride), &pmap, &full[st], u0, bs, i);
    };
    if (threadIdx.x == 0)
        for (int i = 0; i < kSaaStages && i < P; ++i) issue(i, i);
    __syncthreads();
    float hi[kSaaRows / 8][kSaaSlices], lo[kSaaRows / 8][kSaaSlices];
#pragma unroll
    for (int m = 0; m < kSaaRows / 8; ++m)
#pragma unroll
        for (int kk = 0; kk < kSaaSlices; ++kk) hi[m][kk] = lo[m][kk] = 0.f;
    int err = 0, i = 0;
    for (; i < P; ++i) {
        const int st = i % kSaaStages;
        if (!kvtma::mbar_wait_bounded(&full[st], (uint32_t)(i / kSaaStages) & 1u, kSaaWaitPolls)) err |= 1;
        if (err == 0) {
            const float *band = bands + (size_t)st * (stage_stride / 4);
            const int rel = v0 + warp - bstart[st];
#pragma unroll
            for (int kk = 0; kk < kSaaSlices; ++kk) {
                if (kk >= kn) break;
                const int r0 = rel + sh[kk * P + i];
#pragma unroll
                for (int m = 0; m < kSaaRows / 8; ++m) {
                    const int r = r0 + 8 * m;
                    if ((unsigned)r >= (unsigned)nb) {   // outside the band: never expected
                        err |= 4;
                        continue;
                    }
                    const float x = band[r * 32 + lane];
                    const float sm = hi[m][kk] + x;                 // TwoSum(hi, x)
                    const float bp = sm - hi[m][kk];
                    const float e = (hi[m][kk] - (sm - bp)) + (x - bp);
                    hi[m][kk] = sm;
                    lo[m][kk] += e;
                }
            }
        }
        if (__syncthreads_or(err)) break;
        if (threadIdx.x == 0 && i + kSaaStages < P) issue(i + kSaaStages, st);
    }
    if (i < P) {   // failed: record, let the loads in flight land, leave
        if (err) atomicOr(status, err);
        if (threadIdx.x == 0)
            for (int j = i; j < min(P, i + kSaaStages); ++j)
                kvtma::mbar_wait_bounded(&full[j % kSaaStages], (uint32_t)(j / kSaaStages) & 1u, kSaaWaitPolls);
        return;
    }
    const int u = u0 + lane;
    if (u >= nu) return;
    const double w = 1.0 / (double)P;
#pragma unroll
    for (int kk = 0; kk < kSaaSlices; ++kk) {
        if (kk >= kn) break;
#pragma unroll
        for (int m = 0; m < kSaaRows / 8; ++m) {
            const int v = v0 + warp + 8 * m;
            if (v < nv) out[((size_t)(k0 + kk) * nv + v) * nu + u] = (float)(((double)hi[m][kk] + (double)lo[m][kk]) * w);
        }
    }
}

// The learned warm start's elementwise steps.
// ratio = a1 > 0 ? p / a1 : 0, and per block the FP64 sums of (a1 - p)^2 and
// p^2 (the uniform start's data residual: its forward projection is a1).
__global__ void __launch_bounds__(256) warm_ratio_kernel(const float *__restrict__ p, const float *__restrict__ a1,
                                                         float *__restrict__ ratio, size_t n, double *partials) {
    double d0 = 0.0, d1 = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float pv = p[i], av = a1[i];
        ratio[i] = av > 0.f ? pv / av : 0.f;
        const double d = (double)av - (double)pv;
        d0 += d * d;
        d1 += (double)pv * (double)pv;
    }
    for (int o = 16; o > 0; o >>= 1) {
        d0 += __shfl_xor_sync(0xffffffffu, d0, o);
        d1 += __shfl_xor_sync(0xffffffffu, d1, o);
    }
    __shared__ double red[2][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[0][warp] = d0;
        red[1][warp] = d1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            s0 += red[0][w];
            s1 += red[1][w];
        }
        partials[2 * blockIdx.x] = s0;
        partials[2 * blockIdx.x + 1] = s1;
    }
}

// out[0..1] = the sums of the per-block partial pairs (one block, fixed order)
__global__ void sum_pairs_kernel(const double *partials, int nblocks, double *out) {
    __shared__ double sh[2][256];
    double s0 = 0.0, s1 = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        s0 += partials[2 * b];
        s1 += partials[2 * b + 1];
    }
    sh[0][threadIdx.x] = s0;
    sh[1][threadIdx.x] = s1;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sh[0][0];
        out[1] = sh[1][0];
    }
}

// out = sens > 0 ? b / sens (in FP64, rounded once) : 0
__global__ void warm_normalize_kernel(const float *__restrict__ b, const double *__restrict__ sens,
                                      float *__restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double sv = sens[i];
        out[i] = sv > 0.0 ? (float)((double)b[i] / sv) : 0.f;
    }
}

// out = seen ? max(net, eps) : max(saa, eps)
__global__ void warm_fill_kernel(const float *__restrict__ net, const float *__restrict__ saa,
                                 const uint8_t *__restrict__ seen, float eps, float *__restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = fmaxf(seen[i] ? net[i] : saa[i], eps);
}

__global__ void fill_kernel(float *p, size_t n, float v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

template <typename T>
__global__ void to_storage_kernel(const float *in, T *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        Store<T>::st(out + i, in[i]);
}

template <typename T>
__global__ void from_storage_kernel(const T *in, float *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = Store<T>::ld_rw(in + i);
}

// Ellipsoid phantom sampled at voxel centres.  params: n rows of 16 floats =
// centre[3], semi-axes[3], M[9] (local = M (q - c)), density.  The float
// operations and their order are fixed (explicit round-to-nearest
// intrinsics), so the result is bit-identical on every build.
__global__ void __launch_bounds__(256) phantom_kernel(int nx, int ny, int nz, float dx, float dy,
                                                      float dz, const float *__restrict__ params,
                                                      int n, float *__restrict__ vol) {
    extern __shared__ float sp[];
    for (int t = threadIdx.x; t < 16 * n; t += blockDim.x) sp[t] = params[t];
    __syncthreads();
    const size_t plane = (size_t)nx * ny, total = plane * nz;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int z = (int)(idx / plane);
        const size_t rem = idx % plane;
        const int y = (int)(rem / nx), x = (int)(rem % nx);
        const float q0 = __fsub_rn(__fmul_rn(__fadd_rn((float)x, 0.5f), dx), __fmul_rn(__fmul_rn(0.5f, (float)nx), dx));
        const float q1 = __fsub_rn(__fmul_rn(__fadd_rn((float)y, 0.5f), dy), __fmul_rn(__fmul_rn(0.5f, (float)ny), dy));
        const float q2 = __fsub_rn(__fmul_rn(__fadd_rn((float)z, 0.5f), dz), __fmul_rn(__fmul_rn(0.5f, (float)nz), dz));
        float val = 0.f;
        for (int e = 0; e < n; ++e) {
            const float *p = sp + 16 * e;
            const float r0 = __fsub_rn(q0, p[0]), r1 = __fsub_rn(q1, p[1]), r2 = __fsub_rn(q2, p[2]);
            const float l0 = __fadd_rn(__fadd_rn(__fmul_rn(p[6], r0), __fmul_rn(p[7], r1)), __fmul_rn(p[8], r2));
            const float l1 = __fadd_rn(__fadd_rn(__fmul_rn(p[9], r0), __fmul_rn(p[10], r1)), __fmul_rn(p[11], r2));
            const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(p[12], r0), __fmul_rn(p[13], r1)), __fmul_rn(p[14], r2));
            const float t0 = __fdiv_rn(l0, p[3]), t1 = __fdiv_rn(l1, p[4]), t2 = __fdiv_rn(l2, p[5]);
            const float s = __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(t1, t1)), __fmul_rn(t2, t2));
            if (s <= 1.f) val = __fadd_rn(val, p[15]);
        }
        vol[idx] = val;
    }
}

// FP64 reduction of {sum (q-p)^2, sum p^2, sum p log q - q} over n rays:
// grid-stride per-thread sums, one partial triple per block, then a single
// block adds the partials in a fixed order (deterministic).
__global__ void __launch_bounds__(256) residual_partials_kernel(const float *__restrict__ q,
                                                                const float *__restrict__ p, size_t n,
                                                                double *__restrict__ partials) {
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float qi = q[i], pi = p[i];
        const double dq = (double)qi - (double)pi;
        d0 += dq * dq;
        d1 += (double)pi * (double)pi;
        d2 += (qi > 0.f ? (double)pi * (double)logf(qi) : 0.0) - (double)qi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        d0 += __shfl_xor_sync(0xffffffffu, d0, o);
        d1 += __shfl_xor_sync(0xffffffffu, d1, o);
        d2 += __shfl_xor_sync(0xffffffffu, d2, o);
    }
    __shared__ double sh[3][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sh[0][warp] = d0; sh[1][warp] = d1; sh[2][warp] = d2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s0 += sh[0][w]; s1 += sh[1][w]; s2 += sh[2][w]; }
        partials[3 * blockIdx.x] = s0;
        partials[3 * blockIdx.x + 1] = s1;
        partials[3 * blockIdx.x + 2] = s2;
    }
}

__global__ void sum_partials_kernel(const double *__restrict__ partials, int nblocks, double *__restrict__ out) {
    __shared__ double sh[3][256];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        s0 += partials[3 * b];
        s1 += partials[3 * b + 1];
        s2 += partials[3 * b + 2];
    }
    sh[0][threadIdx.x] = s0;
    sh[1][threadIdx.x] = s1;
    sh[2][threadIdx.x] = s2;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
            sh[2][threadIdx.x] += sh[2][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = sh[0][0]; out[1] = sh[1][0]; out[2] = sh[2][0]; }
}

int grid_for(const kv_ctx *ctx, size_t n, int block) {
    size_t g = (n + block - 1) / block;
    size_t cap = (size_t)ctx->sm_count * 8;
    if (cap == 0) cap = 1024;
    return (int)(g < cap ? (g == 0 ? 1 : g) : cap);
}

}  // namespace

// Ramp filtering of the projections along v (the tube's sweep direction)
// for the filtered backprojection: out[p][v][u] = sum_{|k|<=K} h[|k|] *
// in[p][v-k][u], zero outside the detector.  h is the Shepp-Logan kernel
// h[n] = -2 / (pi^2 (4 n^2 - 1)) in pixel units (L. A. Shepp, B. F. Logan,
// IEEE Trans. Nucl. Sci. 21, 1974), truncated at |n| <= K and passed by
// value.  A block holds 32 columns and 32 output rows; the 32 + 2K input
// rows it needs are staged in shared memory (zeros outside the detector),
// and each thread sums the symmetric taps pairwise in FP32.
namespace {

struct RampTaps {
    float h[KV_FBP_MAX_HALF_TAPS + 1];
};

constexpr int kRampRows = 32;

__global__ void __launch_bounds__(256) ramp_v_kernel(const float *__restrict__ in, float *__restrict__ out, int nu,
                                                     int nv, int K, const RampTaps taps) {
    extern __shared__ float tile[];   // [kRampRows + 2K][32]
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int u = blockIdx.x * 32 + tx;
    const int v0 = blockIdx.y * kRampRows;
    const size_t base = (size_t)blockIdx.z * nv * nu;
    const int rows = kRampRows + 2 * K;
    for (int r = ty; r < rows; r += blockDim.y) {
        const int v = v0 - K + r;
        tile[r * 32 + tx] = (u < nu && v >= 0 && v < nv) ? __ldg(in + base + (size_t)v * nu + u) : 0.f;
    }
    __syncthreads();
    if (u >= nu) return;
    for (int o = ty; o < kRampRows; o += blockDim.y) {
        const int v = v0 + o;
        if (v >= nv) break;
        const float *c = tile + (o + K) * 32 + tx;     // input row v
        float acc = taps.h[0] * c[0];
        for (int k = 1; k <= K; ++k) acc = fmaf(taps.h[k], c[-k * 32] + c[k * 32], acc);
        out[base + (size_t)v * nu + u] = acc;
    }
}

}  // namespace

kv_status ramp_filter_launch(kv_plan *plan, const float *in, float *out, int half_taps) {
    const kv_geometry &g = plan->g;
    RampTaps taps;
    for (int n = 0; n <= half_taps; ++n)
        taps.h[n] = (float)(-2.0 / (M_PI * M_PI * (4.0 * (double)n * n - 1.0)));
    const size_t smem = (size_t)(kRampRows + 2 * half_taps) * 32 * sizeof(float);
    KV_CHECK_CUDA(plan->ctx, cudaFuncSetAttribute(ramp_v_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)smem));
    dim3 block(32, 8), grid((g.nu + 31) / 32, (g.nv + kRampRows - 1) / kRampRows, g.n_views);
    LaunchTimer lt(plan->ctx, "ramp_v");
    ramp_v_kernel<<<grid, block, smem, plan->ctx->stream>>>(in, out, g.nu, g.nv, half_taps, taps);
    KV_CHECK_LAUNCH(plan->ctx, "ramp_v_kernel");
    return KV_OK;
}

namespace {

// Rows of the band a block of the staged kernel needs: kSaaRows + the
// largest spread of one block's shifts over its slices, for any view.
int saa_band_rows(const kv_geometry &g, const int32_t *sh) {
    int span = 0;
    for (int k0 = 0; k0 < g.nz; k0 += kSaaSlices)
        for (int i = 0; i < g.n_views; ++i) {
            int lo = sh[(size_t)k0 * g.n_views + i], hi = lo;
            for (int k = k0 + 1; k < std::min(g.nz, k0 + kSaaSlices); ++k) {
                lo = std::min(lo, sh[(size_t)k * g.n_views + i]);
                hi = std::max(hi, sh[(size_t)k * g.n_views + i]);
            }
            span = std::max(span, hi - lo);
        }
    return kSaaRows + span;
}

}  // namespace

kv_status saa_launch(kv_plan *plan, const int32_t *d_shift, const int32_t *h_shift, const float *proj, float *out) {
    const kv_geometry &g = plan->g;
    kv_ctx *ctx = plan->ctx;
    // the staged kernel where its band fits and TMA can address the stack
    const int nb = saa_band_rows(g, h_shift);
    const uint32_t stride = (uint32_t)((32u * nb * 4u + 127u) / 128u * 128u);
    const size_t smem = (size_t)kSaaStages * stride + (size_t)kSaaSlices * g.n_views * sizeof(int32_t) + 128;
    if (nb <= 256 && smem <= 160 * 1024 && (g.nu * 4) % 16 == 0 && reinterpret_cast<uintptr_t>(proj) % 16 == 0 &&
        kvtma::encoder() != nullptr) {
        CUtensorMap map;
        cuuint64_t dims[3] = {(cuuint64_t)g.nu, (cuuint64_t)g.nv, (cuuint64_t)g.n_views};
        cuuint64_t strides[2] = {(cuuint64_t)g.nu * 4, (cuuint64_t)g.nu * g.nv * 4};
        cuuint32_t box[3] = {32, (cuuint32_t)nb, 1};
        cuuint32_t es[3] = {1, 1, 1};
        if (kvtma::encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(proj), dims, strides, box,
                             es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS) {
            KV_CHECK_CUDA(ctx, cudaFuncSetAttribute(saa_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            dim3 grid((g.nu + 31) / 32, (g.nv + kSaaRows - 1) / kSaaRows, (g.nz + kSaaSlices - 1) / kSaaSlices);
            LaunchTimer lt(ctx, "saa");
            saa_band_kernel<<<grid, 256, smem, ctx->stream>>>(map, g.nu, g.nv, g.nz, g.n_views, d_shift, out, nb,
                                                              stride, ctx->d_status);
            KV_CHECK_LAUNCH(ctx, "saa_band_kernel");
            return KV_OK;
        }
    }
    const int kb = 8;
    dim3 block(32, 8), grid((g.nu + 31) / 32, (g.nv + 7) / 8, (g.nz + kb - 1) / kb);
    size_t smem1 = (size_t)kb * g.n_views * sizeof(int32_t);
    if (smem1 > 48 * 1024) return kv_fail(ctx, KV_ERR_UNSUPPORTED, "shift-and-add: too many views");
    LaunchTimer lt(ctx, "saa");
    saa_kernel<<<grid, block, smem1, ctx->stream>>>(g.nu, g.nv, g.nz, g.n_views, d_shift, proj, out, kb);
    KV_CHECK_LAUNCH(ctx, "saa_kernel");
    return KV_OK;
}

kv_status fill_launch(kv_ctx *ctx, float *p, size_t n, float v) {
    LaunchTimer lt(ctx, "fill");
    fill_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(p, n, v);
    KV_CHECK_LAUNCH(ctx, "fill_kernel");
    return KV_OK;
}

kv_status convert_launch(kv_ctx *ctx, const float *in, void *out, size_t n, kv_storage s) {
    int gb = grid_for(ctx, n, 256);
    LaunchTimer lt(ctx, "to_storage");
    if (s == KV_STORAGE_BF16) to_storage_kernel<__nv_bfloat16><<<gb, 256, 0, ctx->stream>>>(in, (__nv_bfloat16 *)out, n);
    else if (s == KV_STORAGE_F16) to_storage_kernel<__half><<<gb, 256, 0, ctx->stream>>>(in, (__half *)out, n);
    else to_storage_kernel<float><<<gb, 256, 0, ctx->stream>>>(in, (float *)out, n);
    KV_CHECK_LAUNCH(ctx, "to_storage_kernel");
    return KV_OK;
}

kv_status convert_back_launch(kv_ctx *ctx, const void *in, float *out, size_t n, kv_storage s) {
    int gb = grid_for(ctx, n, 256);
    LaunchTimer lt(ctx, "from_storage");
    if (s == KV_STORAGE_BF16) from_storage_kernel<__nv_bfloat16><<<gb, 256, 0, ctx->stream>>>((const __nv_bfloat16 *)in, out, n);
    else if (s == KV_STORAGE_F16) from_storage_kernel<__half><<<gb, 256, 0, ctx->stream>>>((const __half *)in, out, n);
    else from_storage_kernel<float><<<gb, 256, 0, ctx->stream>>>((const float *)in, out, n);
    KV_CHECK_LAUNCH(ctx, "from_storage_kernel");
    return KV_OK;
}

kv_status phantom_launch(kv_ctx *ctx, int nx, int ny, int nz, float dx, float dy, float dz,
                         const float *d_params, int n, float *vol) {
    size_t smem = (size_t)16 * n * sizeof(float);
    if (smem > 200 * 1024) return kv_fail(ctx, KV_ERR_INVALID_ARG, "phantom: too many ellipsoids");
    if (smem > 48 * 1024)
        KV_CHECK_CUDA(ctx, cudaFuncSetAttribute(phantom_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    size_t total = (size_t)nx * ny * nz;
    LaunchTimer lt(ctx, "phantom");
    phantom_kernel<<<grid_for(ctx, total, 256), 256, smem, ctx->stream>>>(nx, ny, nz, dx, dy, dz, d_params, n, vol);
    KV_CHECK_LAUNCH(ctx, "phantom_kernel");
    return KV_OK;
}

kv_status residual_reduce_launch(kv_ctx *ctx, const float *q, const float *p, size_t n, double *red) {
    const int nblocks = ctx->sm_count > 0 ? ctx->sm_count * 4 : 512;
    double *partials = nullptr;
    KV_CHECK_CUDA(ctx, cudaMallocAsync((void **)&partials, (size_t)nblocks * 3 * sizeof(double), ctx->stream));
    {
        LaunchTimer lt(ctx, "residual_partials");
        residual_partials_kernel<<<nblocks, 256, 0, ctx->stream>>>(q, p, n, partials);
    }
    {
        LaunchTimer lt(ctx, "sum_partials");
        sum_partials_kernel<<<1, 256, 0, ctx->stream>>>(partials, nblocks, red);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(partials, ctx->stream);
    if (e != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "residual reduction: %s", cudaGetErrorString(e));
    return KV_OK;
}

// ---------------------------------------------------------------------------
// The learned warm start's elementwise steps (device buffers)
// ---------------------------------------------------------------------------

extern "C" kv_status kv_warm_ratio(kv_ctx *ctx, const float *p, const float *a1, float *ratio, size_t n,
                                   double *uniform_residual) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (p == nullptr || a1 == nullptr || ratio == nullptr || n == 0)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_warm_ratio: null buffer or empty");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    const int blocks = grid_for(ctx, n, 256);
    double *partials = nullptr;
    KV_CHECK_CUDA(ctx, cudaMallocAsync((void **)&partials, 2 * sizeof(double) * blocks, ctx->stream));
    {
        LaunchTimer lt(ctx, "warm_ratio");
        warm_ratio_kernel<<<blocks, 256, 0, ctx->stream>>>(p, a1, ratio, n, partials);
        sum_pairs_kernel<<<1, 256, 0, ctx->stream>>>(partials, blocks, ctx->d_red);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(partials, ctx->stream);
    if (e != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "kv_warm_ratio: %s", cudaGetErrorString(e));
    if (uniform_residual != nullptr) {
        double h[2];
        KV_CHECK_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_red, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
        KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *uniform_residual = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    }
    return KV_OK;
}

extern "C" kv_status kv_warm_normalize(kv_ctx *ctx, const float *b, const double *sens, float *out, size_t n) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (b == nullptr || sens == nullptr || out == nullptr || n == 0)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_warm_normalize: null buffer or empty");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    LaunchTimer lt(ctx, "warm_normalize");
    warm_normalize_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(b, sens, out, n);
    KV_CHECK_LAUNCH(ctx, "warm_normalize_kernel");
    return KV_OK;
}

extern "C" kv_status kv_warm_fill(kv_ctx *ctx, const float *net, const float *saa, const uint8_t *seen, float eps,
                                  float *out, size_t n) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (net == nullptr || saa == nullptr || seen == nullptr || out == nullptr || n == 0)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_warm_fill: null buffer or empty");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    LaunchTimer lt(ctx, "warm_fill");
    warm_fill_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(net, saa, seen, eps, out, n);
    KV_CHECK_LAUNCH(ctx, "warm_fill_kernel");
    return KV_OK;
}
