// kv_back_stage.cu -- the EXACT gather backprojector with each view's
// detector patch staged in shared memory by TMA (FP32 storage).
//
// The decomposition and the arithmetic are those of exact_back_r_kernel
// (kv_exact.cu) with one slice per CTA: lanes = 32 voxel columns, warp w =
// voxel rows w, w + 8, ... (R per thread).  Per view, each lane holds the
// x-intervals of its voxel column's candidate detector columns in registers
// (shared by its R rows); the candidate detector rows of the R voxel rows go
// to shared memory as t-intervals, filled side by side; then every
// (candidate row, candidate column) pair is evaluated in lockstep over the R
// rows.  The difference is where the detector values come from: the patch of
// the view that the CTA's voxels can see -- a box of BU x BV pixels, placed
// per view, sized on the host for the worst view and voxel tile -- is loaded
// by cp.async.bulk.tensor into a ring of shared-memory stages one view
// ahead, so the pair loop reads shared memory instead of waiting on L2.
// Weights, and their order per voxel, are exactly those of
// exact_back_r_kernel: the volumes are bit-identical.
#include "kv_internal.h"
#include "kv_exact_common.cuh"
#include "kv_tma.cuh"

#include <string>

namespace {

constexpr int kThreads = 256;           // 8 warps
constexpr int kMaxStages = 3;
constexpr int kSlots = 8;               // candidate columns a lane holds in registers at once
constexpr uint32_t kWaitPolls = 1u << 22;

struct StageArgs {
    int BU, BV, stages;
    uint32_t stage_elems;               // floats between stages (BU * BV rounded up to 128 bytes)
    uint32_t stage_bytes;               // bytes one box load delivers: BU * BV * 4
    uint32_t org_off;                   // byte offset of the per-view patch origins
    int *status;                        // error bits (0: fine)
};

// The candidate detector indices along one axis of the voxels lo .. hi of a
// tile, between the planes with coefficients (a0, b0) and (a1, b1): the first
// candidate of voxel lo and the last of voxel hi.  Both grow with the voxel
// index (b > 0), and these are the backprojector's own expressions, so the
// span holds every candidate any voxel of the tile evaluates.
__host__ __device__ __forceinline__ void cand_span(float a0, float b0, float a1, float b1, int lo, int hi, int n,
                                                   int &c0, int &c1) {
    const float l0 = fminf(((float)lo - a0) * b0, ((float)lo - a1) * b1);
    const float h0 = fmaxf(((float)(lo + 1) - a0) * b0, ((float)(lo + 1) - a1) * b1);
    c0 = max(0, (int)ceilf(fminf(l0, h0) - 0.01f));
    const float l1 = fminf(((float)hi - a0) * b0, ((float)hi - a1) * b1);
    const float h1 = fmaxf(((float)(hi + 1) - a0) * b0, ((float)(hi + 1) - a1) * b1);
    c1 = min(n - 1, (int)floorf(fmaxf(l1, h1) + 0.01f));
}

// One chunk of NS candidate columns (ub .. ub + NS - 1) for the R voxels of
// this thread; rows c < nvc of the staged patch (row stride BU).  The same
// expressions, in the same order, as back_chunk_r in kv_exact.cu.
template <int NS, int R>
__device__ __forceinline__ void stage_chunk(const float4 *xtp, const int *xip, float htop, int i, int ub, int u1,
                                            const float *const (&rowp)[R], int stride, int nvc,
                                            const float2 (*ys)[32], float *acc) {
    float lox[NS], hix[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        lox[s] = 1.f;
        hix[s] = 0.f;
        const int u = ub + s;
        if (u <= u1) {
            const float4 X = xtp[u];
            const int ib = xip[u];
            const float ftx = __fmaf_rn(X.y, htop, X.x);
            const float fi = (float)(i - ib);
            const float ta = cross_tf(fi, ftx, X.z), tb = cross_tf(__fadd_rn(fi, 1.f), ftx, X.z);
            lox[s] = fmaxf(0.f, fminf(ta, tb));
            hix[s] = fminf(1.f, fmaxf(ta, tb));
        }
    }
    for (int c = 0; c < nvc; ++c) {
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const float2 yi = ys[q][c];
            const float *row = rowp[q] + c * stride;
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                const float w = __fsub_rn(fminf(hix[s], yi.y), fmaxf(lox[s], yi.x));
                if (w > 0.f) acc[q] = fmaf(w, row[s], acc[q]);
            }
        }
    }
}

template <int R>
__global__ void __launch_bounds__(kThreads) exact_back_stage_kernel(const __grid_constant__ CUtensorMap pmap,
                                                                    const ExGeom G, const ExactTables T,
                                                                    const BackArgs a, int z0, int mode,
                                                                    const StageArgs A) {
    constexpr int CW = 32 / R;                 // candidates of one voxel row filled per pass
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k = z0 + (int)blockIdx.x;        // slices vary fastest over the grid
    const int i0 = (int)blockIdx.z * 32, j0 = (int)blockIdx.y * 8 * R;
    const int i = i0 + lane;
    const int jw = j0 + warp;                  // voxel row of q = 0; rows jw + 8q
    const int qf = lane / CW, cf = lane % CW;  // this lane fills candidate cf (+ CW f) of row qf
    const int jf = jw + 8 * qf;
    const bool live_i = i < G.nx;

    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[kMaxStages];
    __shared__ float2 ysh[8][R][32];
    // TMA writes its boxes to 128-byte aligned shared memory: the stages start
    // at the first such address of the dynamic region (128 bytes of slack are
    // part of its size) and lie a multiple of 128 bytes apart
    unsigned char *base = smem + ((128u - (kvtma::smem_u32(smem) & 127u)) & 127u);
    float *patch = reinterpret_cast<float *>(base);
    int4 *org = reinterpret_cast<int4 *>(base + A.org_off);   // [n_views]: {u origin, v origin, fits, 0}

    // every view's patch origin, placed once before any load or read of it
    {
        const int i1 = min(i0 + 31, G.nx - 1), j1 = min(j0 + 8 * R - 1, G.ny - 1);
        for (int p = threadIdx.x; p < G.n_views; p += kThreads) {
            const float4 r0 = T.rng[(size_t)p * (G.nz + 1) + k];
            const float4 r1 = T.rng[(size_t)p * (G.nz + 1) + k + 1];
            int ua, ub, va, vb;
            cand_span(r0.x, r0.y, r1.x, r1.y, i0, i1, G.nu, ua, ub);
            cand_span(r0.z, r0.w, r1.z, r1.w, j0, j1, G.nv, va, vb);
            const int x0 = ua & ~3;            // 16-byte aligned start column
            const bool fits = ub - x0 < A.BU && vb - va < A.BV;
            org[p] = make_int4(x0, va, fits ? 1 : 0, 0);
        }
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < A.stages; ++s) kvtma::mbar_init(&full[s], 1);
        kvtma::fence_mbar_init();
    }
    __syncthreads();
    // thread 0: load view p's patch into stage st
    auto issue = [&](int p, int st) {
        kvtma::fence_proxy_async_smem();
        kvtma::mbar_arrive_expect_tx(&full[st], A.stage_bytes);
        kvtma::tma_load_3d(kvtma::smem_u32(patch + (size_t)st * A.stage_elems), &pmap, &full[st], org[p].x,
                           org[p].y, p);
    };
    if (threadIdx.x == 0)
        for (int p = 0; p < A.stages && p < G.n_views; ++p) issue(p, p);

    float acc[R];
#pragma unroll
    for (int q = 0; q < R; ++q) acc[q] = 0.f;
    int err = 0;
    int p = 0;
    for (; p < G.n_views; ++p) {
        const int st = p % A.stages;
        if (!kvtma::mbar_wait_bounded(&full[st], (uint32_t)(p / A.stages) & 1u, kWaitPolls)) err |= 8;
        const int4 o = org[p];
        if (!o.z) err |= 16;
        if (err == 0) {
            const float *img = patch + (size_t)st * A.stage_elems;
            const float htop = T.hr[(size_t)p * (G.nz + 1) + k + 1];
            const float4 r0 = T.rng[(size_t)p * (G.nz + 1) + k];
            const float4 r1 = T.rng[(size_t)p * (G.nz + 1) + k + 1];
            const float4 *xtp = T.xt + (size_t)p * G.nu;
            const int *xip = T.xi + (size_t)p * G.nu;
            // candidate detector columns of voxel column i (per lane)
            const float ulo = fminf(((float)i - r0.x) * r0.y, ((float)i - r1.x) * r1.y);
            const float uhi = fmaxf(((float)(i + 1) - r0.x) * r0.y, ((float)(i + 1) - r1.x) * r1.y);
            const int u0 = max(0, (int)ceilf(fminf(ulo, uhi) - 0.01f));
            int u1 = min(G.nu - 1, (int)floorf(fmaxf(ulo, uhi) + 0.01f));
            if (!live_i) u1 = u0 - 1;
            const int n_u_warp = __reduce_max_sync(0xffffffffu, u1 >= u0 ? u1 - u0 + 1 : 0);
            // candidate detector rows of the lane's fill row
            int v0f = 0, nvf = 0;
            if (jf < G.ny) {
                const float vlo = fminf(((float)jf - r0.z) * r0.w, ((float)jf - r1.z) * r1.w);
                const float vhi = fmaxf(((float)(jf + 1) - r0.z) * r0.w, ((float)(jf + 1) - r1.z) * r1.w);
                v0f = max(0, (int)ceilf(fminf(vlo, vhi) - 0.01f));
                const int v1 = min(G.nv - 1, (int)floorf(fmaxf(vlo, vhi) + 0.01f));
                nvf = max(0, v1 - v0f + 1);
            }
            const int nvmax = __reduce_max_sync(0xffffffffu, nvf);
            int v0[R];
#pragma unroll
            for (int q = 0; q < R; ++q) v0[q] = __shfl_sync(0xffffffffu, v0f, q * CW);
            for (int vb = 0; vb < nvmax; vb += 32) {
                const int nvc = min(32, nvmax - vb);
                for (int f = 0; f * CW < nvc; ++f) {
                    float2 iv = make_float2(1.f, 0.f);
                    const int c = vb + f * CW + cf;
                    if (c < nvf) {
                        const int vv = v0f + c;
                        const float4 Y = T.yt[(size_t)p * G.nv + vv];
                        const int jb = T.yi[(size_t)p * G.nv + vv];
                        const float fty = __fmaf_rn(Y.y, htop, Y.x);
                        const float fj = (float)(jf - jb);
                        const float ta = cross_tf(fj, fty, Y.z), tb = cross_tf(__fadd_rn(fj, 1.f), fty, Y.z);
                        iv = make_float2(fmaxf(0.f, fminf(ta, tb)), fminf(1.f, fmaxf(ta, tb)));
                    }
                    ysh[warp][qf][f * CW + cf] = iv;
                }
                __syncwarp();
                for (int cb = 0; cb * kSlots < n_u_warp; ++cb) {
                    const int ub = u0 + cb * kSlots;
                    const int nslot = min(kSlots, n_u_warp - cb * kSlots);
                    // patch-relative row starts (rows and columns the weights
                    // reach lie inside the patch; the rest are never read)
                    const float *rowp[R];
#pragma unroll
                    for (int q = 0; q < R; ++q) rowp[q] = img + (v0[q] + vb - o.y) * A.BU + (ub - o.x);
                    switch (nslot) {
                    case 1: stage_chunk<1, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    case 2: stage_chunk<2, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    case 3: stage_chunk<3, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    case 4: stage_chunk<4, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    case 5: stage_chunk<5, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    case 6: stage_chunk<6, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    case 7: stage_chunk<7, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    default: stage_chunk<8, R>(xtp, xip, htop, i, ub, u1, rowp, A.BU, nvc, ysh[warp], acc); break;
                    }
                }
                __syncwarp();
            }
        }
        // every warp is done with stage st: refill it with view p + stages
        if (__syncthreads_or(err)) break;
        if (threadIdx.x == 0 && p + A.stages < G.n_views) issue(p + A.stages, st);
    }
    if (p < G.n_views) {
        // failed: record, let the loads still in flight land, and leave
        if (err) atomicOr(A.status, err);
        if (threadIdx.x == 0)
            for (int j = p; j < min(G.n_views, p + A.stages); ++j)
                kvtma::mbar_wait_bounded(&full[j % A.stages], (uint32_t)(j / A.stages) & 1u, kWaitPolls);
        return;
    }
    if (!live_i) return;
    float *vol = static_cast<float *>(a.vol);
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const int j = jw + 8 * q;
        if (j >= G.ny) continue;
        const size_t idx = ((size_t)k * G.ny + j) * G.nx + i;
        const float b = acc[q];
        if (mode == BACK_PLAIN) {
            vol[idx] = b;
        } else if (mode == BACK_MLEM) {
            const double sv = a.sens[idx];
            if (sv > 0.0) vol[idx] = (float)((double)vol[idx] * (double)b / sv);
        } else if (mode == BACK_SART) {
            const double sv = a.sens[idx];
            if (sv > 0.0) vol[idx] = vol[idx] + (float)((double)(a.relax * b) / sv);
        }
    }
}

struct StageLayout {
    uint32_t stage_stride, org_off;
    size_t total;
};

StageLayout stage_layout(int stages, int BU, int BV, int n_views) {
    auto up = [](size_t v, size_t al) { return (v + al - 1) / al * al; };
    StageLayout L;
    L.stage_stride = (uint32_t)up((size_t)BU * BV * sizeof(float), 128);
    L.org_off = (uint32_t)((size_t)stages * L.stage_stride);
    L.total = up((size_t)L.org_off + (size_t)n_views * sizeof(int4), 128) + 128;   // + alignment slack
    return L;
}

}  // namespace

bool back_stage_fit(const kv_plan *plan, int R, int stages, BackStageCfg *out, std::string *why) {
    const kv_geometry &g = plan->g;
    const ExactHostTables &H = plan->hx;
    auto no = [&](const char *m) {
        if (why) *why = m;
        return false;
    };
    if (R != 4 && R != 8) return no("staged backprojector: voxel rows per thread must be 4 or 8");
    if (stages < 2 || stages > kMaxStages) return no("staged backprojector: stage count out of range");
    if (plan->storage != KV_STORAGE_F32) return no("staged backprojector: FP32 storage only");
    if (kvtma::encoder() == nullptr) return no("cuTensorMapEncodeTiled is not available");
    if (((size_t)g.nu * sizeof(float)) % 16 != 0) return no("detector rows are not a whole number of 16-byte units");
    if (H.rng.size() != (size_t)g.n_views * (g.nz + 1)) return no("host tables missing");
    const int TV = 8 * R;
    int bu = 0, bv = 0;
    for (int p = 0; p < g.n_views; ++p) {
        for (int k = 0; k < g.nz; ++k) {
            const float4 r0 = H.rng[(size_t)p * (g.nz + 1) + k], r1 = H.rng[(size_t)p * (g.nz + 1) + k + 1];
            for (int i0 = 0; i0 < g.nx; i0 += 32) {
                int ua, ub;
                cand_span(r0.x, r0.y, r1.x, r1.y, i0, std::min(i0 + 31, g.nx - 1), g.nu, ua, ub);
                bu = std::max(bu, ub - (ua & ~3) + 1);
            }
            for (int j0 = 0; j0 < g.ny; j0 += TV) {
                int va, vb;
                cand_span(r0.z, r0.w, r1.z, r1.w, j0, std::min(j0 + TV - 1, g.ny - 1), g.nv, va, vb);
                bv = std::max(bv, vb - va + 1);
            }
        }
    }
    bu = (bu + 3) / 4 * 4;
    if (bu < 4) bu = 4;
    if (bv < 1) bv = 1;
    if (bu > 256 || bv > 256) return no("staged backprojector: a tile sees more than 256 detector columns or rows");
    const StageLayout L = stage_layout(stages, bu, bv, g.n_views);
    if (L.total > 200 * 1024) return no("staged backprojector: the patch stages do not fit in shared memory");
    BackStageCfg c;
    c.R = R;
    c.stages = stages;
    c.BU = bu;
    c.BV = bv;
    c.smem = L.total;
    *out = c;
    return true;
}

kv_status back_stage_launch(kv_plan *plan, BackMode mode, const BackArgs &a, int z0, int nzs, int n_views) {
    const BackStageCfg &c = plan->bstage;
    const kv_geometry &g = plan->g;
    if (reinterpret_cast<uintptr_t>(a.yp) % 16 != 0)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "projection buffer is not 16-byte aligned");
    CUtensorMap map;
    cuuint64_t dims[3] = {(cuuint64_t)g.nu, (cuuint64_t)g.nv, (cuuint64_t)n_views};
    cuuint64_t strides[2] = {(cuuint64_t)g.nu * sizeof(float), (cuuint64_t)g.nu * g.nv * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)c.BU, (cuuint32_t)c.BV, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    if (kvtma::encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(a.yp), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return kv_fail(plan->ctx, KV_ERR_CUDA, "projection tensor map rejected");
    const StageLayout L = stage_layout(c.stages, c.BU, c.BV, n_views);
    StageArgs A;
    A.BU = c.BU;
    A.BV = c.BV;
    A.stages = c.stages;
    A.stage_elems = L.stage_stride / sizeof(float);
    A.stage_bytes = (uint32_t)c.BU * c.BV * sizeof(float);
    A.org_off = L.org_off;
    A.status = plan->ctx->d_status;
    const ExGeom G{g.nx, g.ny, g.nz, g.nu, g.nv, n_views};
    dim3 grid(nzs, (g.ny + 8 * c.R - 1) / (8 * c.R), (g.nx + 31) / 32);
    const void *fn = c.R == 8 ? (const void *)exact_back_stage_kernel<8> : (const void *)exact_back_stage_kernel<4>;
    KV_CHECK_CUDA(plan->ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
    cudaStream_t st = plan->ctx->stream;
    LaunchTimer lt(plan->ctx, "exact_back");
    if (c.R == 8)
        exact_back_stage_kernel<8><<<grid, kThreads, L.total, st>>>(map, G, plan->ex, a, z0, (int)mode, A);
    else
        exact_back_stage_kernel<4><<<grid, kThreads, L.total, st>>>(map, G, plan->ex, a, z0, (int)mode, A);
    KV_CHECK_LAUNCH(plan->ctx, "exact_back_stage_kernel");
    return KV_OK;
}
