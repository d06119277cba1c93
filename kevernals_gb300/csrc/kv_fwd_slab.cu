// kv_fwd_slab.cu -- EXACT forward projector with the volume staged slab by
// slab in shared memory (sm_103a).
//
// A CTA owns a tile of 32 x 8R rays of one view: 32 detector columns (one
// per lane) by 8R detector rows (warp w owns rows w, w + 8, ...).  It walks
// the volume in slabs of S slices.  For every slab, one thread issues a TMA
// load (cp.async.bulk.tensor.3d) of the box of voxels the tile's rays can
// touch in that slab -- BX x BY x S voxels, placed from the tile's corner
// rays -- into a ring of shared-memory stages; voxels outside the volume
// read zeros, so the rays need no bounds checks.  Loads run `stages - 1`
// slabs ahead of the compute.
//
// Within slice k a ray with top-plane position ftx (relative to its column
// base) starts in column fi and meets the column planes at slice-local
// parameters X1 < X2 (cross_tf: the same float expression as the gather
// backprojector's); its row sequence has crossings Y1 < Y2 < ... .  The
// length in (row r, column c) is
//     [min(Y_{r+1}, X_{c+1}) - max(Y_r, X_c)]+      (Y_0 = X_0 = 0, ends clamped to 1)
// which is, bit for bit, the backprojector's min(1, tx_hi, ty_hi) -
// max(0, tx_lo, ty_lo) for that (voxel, ray) pair.  A slice has at most
// three columns and five rows per ray (checked on the host); all pairs are
// evaluated branch-free and only those with a positive length read the box.
//
// The x part (fi, X1, X2) depends on the detector column only and is shared
// by the R rays of a thread; the y part depends on the row only, so it is
// computed once per (row, slice) of the slab into a shared-memory descriptor
// that every lane of the row's warp reads.
//
// Launch order: CTAs of the same detector-row tile of consecutive views run
// together ("view groups"); the volume region those rays cross moves slowly
// from view to view, so one group sweeps the volume through L2 about once.
#include "kv_internal.h"
#include "kv_exact_common.cuh"
#include "kv_tma.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace {

constexpr int kThreads = 256;        // 8 warps
constexpr int kMaxStages = 4;
constexpr int kMaxRows = 5;          // voxel rows one ray meets within one slice
constexpr uint32_t kWaitPolls = 1u << 22;

// Per (detector row, slice) of a slab: the row crossings and where the
// ray's first row sits in the stage.
struct YDesc {
    float4 yc;      // min(1, Y1 .. Y4)
    int rowoff;     // byte offset of (slice, first row) within the stage
    int rowstep;    // +-BX elements, in bytes: next row in the direction of travel
    int nr;         // rows met in this slice (0: no ray)
    int row0;       // volume row of the first row (SART row sums count in-volume voxels only)
};

struct SlabArgs {
    int S, BX, BY, stages, nslab, group, n_ut, n_vt, align;
    uint32_t stage_elems;            // elements between stages (BX * BY * S rounded up to 128 bytes)
    uint32_t stage_bytes;            // bytes one box load delivers: BX * BY * S * element size
    uint32_t desc_off, hr_off, yt_off, yi_off, org_off;   // byte offsets in dynamic shared memory
    int *status;                     // error bits (0: fine)
};

// c - (c mod a) with a non-negative remainder.
__host__ __device__ __forceinline__ int floor_to(int c, int a) {
    int r = c % a;
    if (r < 0) r += a;
    return c - r;
}

// Columns (or rows) met on the planes of heights h0, h1 by the rays of two
// detector columns: floor of the ray position, table base added.
__host__ __device__ __forceinline__ void span2(float4 A, int ia, float4 B, int ibb, float h0, float h1, int &lo,
                                               int &hi) {
    const int c0 = ia + (int)floorf(fmaf(A.y, h0, A.x));
    const int c1 = ia + (int)floorf(fmaf(A.y, h1, A.x));
    const int c2 = ibb + (int)floorf(fmaf(B.y, h0, B.x));
    const int c3 = ibb + (int)floorf(fmaf(B.y, h1, B.x));
    lo = min(min(c0, c1), min(c2, c3));
    hi = max(max(c0, c1), max(c2, c3));
}

// Box origin of slab s for the tile whose corner rays are (Xa, Xb) in x and
// (Ya, Yb) in y: three columns of margin (a ray's start column and the two
// after it stay inside), two rows (the rows a ray meets are exactly those
// between its end planes).  x is rounded down to the TMA's 16-byte grid.
__host__ __device__ __forceinline__ void box_origin(float4 Xa, int ia, float4 Xb, int ibb, float4 Ya, int ja,
                                                    float4 Yb, int jbb, float h0, float h1, int align, int &x0,
                                                    int &y0, int &need_x, int &need_y) {
    int cmin, cmax, rmin, rmax;
    span2(Xa, ia, Xb, ibb, h0, h1, cmin, cmax);
    span2(Ya, ja, Yb, jbb, h0, h1, rmin, rmax);
    x0 = floor_to(cmin - 3, align);
    y0 = rmin - 2;
    need_x = cmax + 3 - x0 + 1;
    need_y = rmax + 2 - y0 + 1;
}

template <typename T> __device__ __forceinline__ float sld(const T *p);
template <> __device__ __forceinline__ float sld<float>(const float *p) { return *p; }
template <> __device__ __forceinline__ float sld<__nv_bfloat16>(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
template <> __device__ __forceinline__ float sld<__half>(const __half *p) { return __half2float(*p); }

// Where the SART row sum may count a length: the voxel lies in the volume
// (the box reads zeros outside it, which adds nothing to the line integral
// but must add nothing to the row sum either).
__device__ __forceinline__ bool in_volume(int col, int row, int nx, int ny) {
    return (unsigned)col < (unsigned)nx && (unsigned)row < (unsigned)ny;
}

// The rays q0 .. q0+NQ-1 of this thread (same detector column, rows 8 apart)
// in one slice, their rows in lockstep: rows past a ray's own count have
// lo = hi = 1 (the crossings are clamped to 1) and weigh nothing, and its
// row address stops advancing there, so every read stays inside the box.
// Lengths in clamp form: with a1 = min(max(X1, lo), hi) and a2 likewise, the
// ray spends a1 - lo in its first column, a2 - a1 in the second and hi - a2
// in the third.  Where min(hi, X_{c+1}) - max(lo, X_c) is positive these are
// the same two floats subtracted (the backprojector's weight, bit for bit);
// where it is not they are zero.  SXC: the column step when every lane of
// the warp moves the same way (+1 / -1: immediate offsets), 0 otherwise.
template <typename VolT, int NQ, bool NC3, bool SART, int SXC>
__device__ __forceinline__ void slice_rays(const unsigned char *box, const YDesc *d8, int colb_bytes, int sx_bytes,
                                           float X1, float X2, float (*acc)[2], float *wsum, int col0, int sx,
                                           int nx, int ny) {
    const int cstep = SXC != 0 ? SXC * (int)sizeof(VolT) : sx_bytes;
    int off[NQ], nr[NQ], step[NQ], row0[NQ];
    float4 yc[NQ];
    float lo[NQ], hi[NQ];
    int nrmax = 0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const YDesc d = d8[8 * q];
        off[q] = d.rowoff + colb_bytes;
        nr[q] = d.nr;
        step[q] = d.rowstep;
        row0[q] = d.row0;
        yc[q] = d.yc;
        lo[q] = 0.f;
        hi[q] = d.yc.x;
        nrmax = max(nrmax, d.nr);
    }
#pragma unroll
    for (int r = 0; r < kMaxRows; ++r) {
        if (r >= nrmax) break;   // warp-uniform
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            if (r > 0) {
                lo[q] = hi[q];
                hi[q] = r == 1 ? yc[q].y : (r == 2 ? yc[q].z : (r == 3 ? yc[q].w : 1.f));
                if (r < nr[q]) off[q] += step[q];
            }
            const float a1 = fminf(fmaxf(X1, lo[q]), hi[q]);
            const float w0 = __fsub_rn(a1, lo[q]);
            float w1, w2 = 0.f;
            if (NC3) {
                const float a2 = fminf(fmaxf(X2, lo[q]), hi[q]);
                w1 = __fsub_rn(a2, a1);
                w2 = __fsub_rn(hi[q], a2);
            } else {
                w1 = __fsub_rn(hi[q], a1);
            }
            acc[q][0] = fmaf(w0, sld(reinterpret_cast<const VolT *>(box + off[q])), acc[q][0]);
            acc[q][1] = fmaf(w1, sld(reinterpret_cast<const VolT *>(box + off[q] + cstep)), acc[q][1]);
            if (NC3) acc[q][0] = fmaf(w2, sld(reinterpret_cast<const VolT *>(box + off[q] + 2 * cstep)), acc[q][0]);
            if (SART) {
                const int row = row0[q] + r * (step[q] > 0 ? 1 : -1);
                float ws = in_volume(col0, row, nx, ny) ? w0 : 0.f;
                if (in_volume(col0 + sx, row, nx, ny)) ws += w1;
                if (NC3 && in_volume(col0 + 2 * sx, row, nx, ny)) ws += w2;
                wsum[q] += ws;
            }
        }
    }
}

template <typename VolT, typename ProjT, int MODE, int R>
__global__ void __launch_bounds__(kThreads, R >= 8 ? 2 : 3) fwd_slab_kernel(const __grid_constant__ CUtensorMap vmap,
                                                            const ExGeom G, const ExactTables T, const FwdArgs a,
                                                            double *partials, const SlabArgs A) {
    constexpr int TV = 8 * R;
    constexpr bool SART = MODE == FWD_SART;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[kMaxStages];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    // ---- tile: detector columns u0 .. u0+31, rows v0 .. v0+TV-1 of view p
    const int ut = (int)(blockIdx.x % (unsigned)A.n_ut);
    const int t = (int)(blockIdx.x / (unsigned)A.n_ut);
    const int per_group = A.group * A.n_vt;
    const int g = t / per_group;
    const int g_first = g * A.group;
    const int g_n = min(A.group, G.n_views - g_first);
    const int loc = t - g * per_group;
    const int vt = loc / g_n;
    const int p = g_first + (loc - vt * g_n);
    const int u0 = ut * 32, v0 = vt * TV;

    // TMA writes its boxes to 128-byte aligned shared memory: the stages start
    // at the first such address of the dynamic region (128 bytes of slack are
    // part of its size) and lie a multiple of 128 bytes apart
    unsigned char *base = smem + ((128u - (kvtma::smem_u32(smem) & 127u)) & 127u);
    VolT *boxes = reinterpret_cast<VolT *>(base);
    YDesc *desc = reinterpret_cast<YDesc *>(base + A.desc_off);       // [2][S][TV]
    float *s_hr = reinterpret_cast<float *>(base + A.hr_off);         // [nz + 1]
    float4 *s_yt = reinterpret_cast<float4 *>(base + A.yt_off);       // [TV]
    int *s_yi = reinterpret_cast<int *>(base + A.yi_off);             // [TV]
    int2 *org = reinterpret_cast<int2 *>(base + A.org_off);           // [nslab]: box origin of each slab

    for (int i = threadIdx.x; i <= G.nz; i += kThreads) s_hr[i] = T.hr[(size_t)p * (G.nz + 1) + i];
    if (threadIdx.x < TV) {
        const int v = min(v0 + (int)threadIdx.x, G.nv - 1);
        s_yt[threadIdx.x] = T.yt[(size_t)p * G.nv + v];
        s_yi[threadIdx.x] = T.yi[(size_t)p * G.nv + v];
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < A.stages; ++s) kvtma::mbar_init(&full[s], 1);
        kvtma::fence_mbar_init();
    }
    __syncthreads();

    // the box of every slab, placed once before any load or row descriptor
    // needs it (a box origin written while the pipeline runs would be read by
    // the next slab's descriptors with no barrier in between at two stages)
    {
        const int ua = u0, ub = min(u0 + 31, G.nu - 1);
        const int vb_local = min(TV - 1, G.nv - 1 - v0);
        for (int s = threadIdx.x; s < A.nslab; s += kThreads) {
            const int ks = s * A.S, ke = min(ks + A.S, G.nz);
            const float4 Xa = T.xt[(size_t)p * G.nu + ua], Xb = T.xt[(size_t)p * G.nu + ub];
            const int ia = T.xi[(size_t)p * G.nu + ua], ibb = T.xi[(size_t)p * G.nu + ub];
            int x0, y0, nxn, nyn;
            box_origin(Xa, ia, Xb, ibb, s_yt[0], s_yi[0], s_yt[vb_local], s_yi[vb_local], s_hr[ks], s_hr[ke],
                       A.align, x0, y0, nxn, nyn);
            org[s] = make_int2(x0, y0);
        }
    }
    __syncthreads();
    // thread 0: load the box of slab s into stage st
    auto issue = [&](int s, int st) {
        kvtma::fence_proxy_async_smem();
        kvtma::mbar_arrive_expect_tx(&full[st], A.stage_bytes);
        kvtma::tma_load_3d(kvtma::smem_u32(boxes + (size_t)st * A.stage_elems), &vmap, &full[st], org[s].x, org[s].y,
                           s * A.S);
    };
    // threads < S*TV: the row descriptors of slab s into buffer buf
    auto make_desc = [&](int s, int buf) -> int {
        const int kk = threadIdx.x / TV, vl = threadIdx.x - kk * TV;
        const int k = s * A.S + kk, v = v0 + vl;
        YDesc d;
        d.yc = make_float4(0.f, 0.f, 0.f, 0.f);   // no ray: every length is zero
        d.rowoff = 0;
        d.rowstep = 0;
        d.nr = 0;
        d.row0 = 0;
        int bad = 0;
        if (k < G.nz && v < G.nv) {
            const float4 Y = s_yt[vl];
            const float fty = __fmaf_rn(Y.y, s_hr[k + 1], Y.x);
            const float fl = floorf(fty);
            const bool negy = Y.z < 0.f;
            const float fj = (negy && fl == fty) ? fl - 1.f : fl;
            const float sy = negy ? -1.f : 1.f;
            const float p1 = __fadd_rn(fj, negy ? 0.f : 1.f);
            const float p2 = __fadd_rn(p1, sy), p3 = __fadd_rn(p2, sy), p4 = __fadd_rn(p3, sy);
            const float y1 = cross_tf(p1, fty, Y.z), y2 = cross_tf(p2, fty, Y.z);
            const float y3 = cross_tf(p3, fty, Y.z), y4 = cross_tf(p4, fty, Y.z);
            const int nr = 1 + (y1 < 1.f) + (y2 < 1.f) + (y3 < 1.f) + (y4 < 1.f);
            const int j0 = s_yi[vl] + (int)fj;
            const int js = j0 - org[s].y;
            const int je = js + (negy ? 1 - nr : nr - 1);
            if (min(js, je) < 0 || max(js, je) >= A.BY) {
                bad = 4;
            } else {
                d.yc = make_float4(fminf(1.f, y1), fminf(1.f, y2), fminf(1.f, y3), fminf(1.f, y4));
                d.rowoff = (kk * A.BY + js) * A.BX * (int)sizeof(VolT);
                d.rowstep = (negy ? -A.BX : A.BX) * (int)sizeof(VolT);
                d.nr = nr;
                d.row0 = j0;
            }
        }
        desc[(buf * A.S + kk) * TV + vl] = d;
        return bad;
    };

    if (threadIdx.x == 0)
        for (int s = 0; s < A.stages && s < A.nslab; ++s) issue(s, s);
    __syncthreads();
    int err = 0;
    if (threadIdx.x < A.S * TV) err |= make_desc(0, 0);
    __syncthreads();

    // ---- this lane's detector column
    const int u = u0 + lane;
    const bool live_u = u < G.nu;
    const int uc = live_u ? u : G.nu - 1;
    const float4 X = T.xt[(size_t)p * G.nu + uc];
    const int ib = T.xi[(size_t)p * G.nu + uc];
    const bool negx = X.z < 0.f;
    const float e1 = negx ? 0.f : 1.f, e2 = negx ? -1.f : 2.f;
    const int sx = negx ? -1 : 1;
    const bool nc3 = __any_sync(0xffffffffu, fabsf(X.z) < 1.f);   // some ray crosses two column planes

    // warp-uniform column direction: immediate offsets when all lanes agree
    const int sxmode = __all_sync(0xffffffffu, sx > 0) ? 1 : (__all_sync(0xffffffffu, sx < 0) ? -1 : 0);
    const int sx_bytes = sx * (int)sizeof(VolT);
    constexpr int NQ = R < 4 ? R : 4;   // rays per lockstep group

    float acc[R][2], wsum[R];
#pragma unroll
    for (int q = 0; q < R; ++q) acc[q][0] = acc[q][1] = wsum[q] = 0.f;

    int s = 0;
    for (; s < A.nslab; ++s) {
        const int st = s % A.stages;
        if (!kvtma::mbar_wait_bounded(&full[st], (uint32_t)(s / A.stages) & 1u, kWaitPolls)) err |= 1;
        if (err == 0) {
            const unsigned char *box = reinterpret_cast<const unsigned char *>(boxes + (size_t)st * A.stage_elems);
            const YDesc *dsc = desc + (s & 1) * A.S * TV;
            const int xoff = ib - org[s].x;
            const int kend = min(A.S, G.nz - s * A.S);
            for (int kk = 0; kk < kend; ++kk) {
                const float ftx = __fmaf_rn(X.y, s_hr[s * A.S + kk + 1], X.x);
                const float fl = floorf(ftx);
                const float fi = (negx && fl == ftx) ? fl - 1.f : fl;
                const float X1 = cross_tf(__fadd_rn(fi, e1), ftx, X.z);
                const float X2 = nc3 ? cross_tf(__fadd_rn(fi, e2), ftx, X.z) : 2.f;
                const int colb = (int)fi + xoff;
                if ((unsigned)(colb - 2) > (unsigned)(A.BX - 5)) {   // outside the box: never expected
                    err |= 2;
                    continue;
                }
                const int colb_bytes = colb * (int)sizeof(VolT);
                const int col0 = (int)fi + ib;
                const YDesc *d8 = dsc + kk * TV + warp;
#pragma unroll
                for (int q0 = 0; q0 < R; q0 += NQ) {
#define KV_SLICE(NC3_, SXC_)                                                                              \
    slice_rays<VolT, NQ, NC3_, SART, SXC_>(box, d8 + 8 * q0, colb_bytes, sx_bytes, X1, X2, acc + q0, wsum + q0, \
                                           col0, sx, G.nx, G.ny)
                    if (nc3) {
                        if (sxmode > 0) KV_SLICE(true, 1);
                        else if (sxmode < 0) KV_SLICE(true, -1);
                        else KV_SLICE(true, 0);
                    } else {
                        if (sxmode > 0) KV_SLICE(false, 1);
                        else if (sxmode < 0) KV_SLICE(false, -1);
                        else KV_SLICE(false, 0);
                    }
#undef KV_SLICE
                }
            }
        }
        if (s + 1 < A.nslab && threadIdx.x < A.S * TV) err |= make_desc(s + 1, (s + 1) & 1);
        if (__syncthreads_or(err)) break;
        if (threadIdx.x == 0 && s + A.stages < A.nslab) issue(s + A.stages, st);
    }
    if (s < A.nslab) {
        // failed: record, let the loads still in flight land, and leave
        if (err) atomicOr(A.status, err);
        if (threadIdx.x == 0)
            for (int j = s; j < min(A.nslab, s + A.stages); ++j)
                kvtma::mbar_wait_bounded(&full[j % A.stages], (uint32_t)(j / A.stages) & 1u, kWaitPolls);
        return;
    }

    // ---- epilogue: line integrals, fused ratio, FP64 reductions
    const float4 VI = T.vinfo[p];
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const int vl = warp + 8 * q, v = v0 + vl;
        if (!live_u || v >= G.nv) continue;
        const float ls = ray_factor(X.w, s_yt[vl].w, VI);
        const float qv = __fadd_rn(acc[q][0], acc[q][1]) * ls;
        const size_t ray = ((size_t)p * G.nv + v) * G.nu + u;
        ProjT *out = static_cast<ProjT *>(a.out);
        float pm = 0.f;
        if (MODE != FWD_PLAIN) pm = Store<ProjT>::ld(static_cast<const ProjT *>(a.meas) + ray);
        if (MODE == FWD_PLAIN) {
            Store<ProjT>::st(out + ray, qv);
        } else if (MODE == FWD_MLEM) {
            const float r = qv > 0.f ? a.relax * pm / qv : 0.f;
            Store<ProjT>::st(out + ray, r * ls);
        } else if (MODE == FWD_SART) {
            const float rows = wsum[q] * ls;
            const float r = rows > 0.f ? (pm - qv) / rows : 0.f;
            Store<ProjT>::st(out + ray, r * ls);
        }
        if (partials != nullptr) {
            const double dq = (double)qv - (double)pm;
            d0 += dq * dq;
            d1 += (double)pm * (double)pm;
            d2 += (qv > 0.f ? (double)pm * (double)logf(qv) : 0.0) - (double)qv;
        }
    }
    if (partials != nullptr) {
        for (int o = 16; o > 0; o >>= 1) {
            d0 += __shfl_xor_sync(0xffffffffu, d0, o);
            d1 += __shfl_xor_sync(0xffffffffu, d1, o);
            d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        }
        __shared__ double red[3][kThreads / 32];
        if (lane == 0) {
            red[0][warp] = d0;
            red[1][warp] = d1;
            red[2][warp] = d2;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double r0 = 0.0, r1 = 0.0, r2 = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) {
                r0 += red[0][w];
                r1 += red[1][w];
                r2 += red[2][w];
            }
            partials[3 * (size_t)blockIdx.x + 0] = r0;
            partials[3 * (size_t)blockIdx.x + 1] = r1;
            partials[3 * (size_t)blockIdx.x + 2] = r2;
        }
    }
}

// Dynamic shared memory layout of one CTA (byte offsets from the first
// 128-byte aligned address of the region).
struct SmemLayout {
    uint32_t stage_stride, desc_off, hr_off, yt_off, yi_off, org_off;
    size_t total;
};

SmemLayout smem_layout(int R, int S, int stages, int BX, int BY, int nz, int es) {
    auto up = [](size_t v, size_t a) { return (v + a - 1) / a * a; };
    const int TV = 8 * R;
    SmemLayout L;
    L.stage_stride = (uint32_t)up((size_t)BX * BY * S * es, 128);
    size_t off = (size_t)stages * L.stage_stride;
    L.desc_off = (uint32_t)off;
    off += (size_t)2 * S * TV * sizeof(YDesc);
    L.hr_off = (uint32_t)off;
    off = up(off + (size_t)(nz + 1) * sizeof(float), 16);
    L.yt_off = (uint32_t)off;
    off += (size_t)TV * sizeof(float4);
    L.yi_off = (uint32_t)off;
    off = up(off + (size_t)TV * sizeof(int), 8);
    L.org_off = (uint32_t)off;
    off += (size_t)((nz + S - 1) / S) * sizeof(int2);
    L.total = up(off, 128) + 128;   // + slack for aligning the region's start
    return L;
}

template <typename VolT, typename ProjT, int R>
kv_status slab_launch_r(kv_plan *plan, const CUtensorMap &map, const ExGeom &G, const ExactTables &t, FwdMode mode,
                        const FwdArgs &a, double *partials, const SlabArgs &A, unsigned grid, size_t smem) {
    cudaStream_t st = plan->ctx->stream;
    const void *fn = nullptr;
    switch (mode) {
    case FWD_PLAIN: fn = (const void *)fwd_slab_kernel<VolT, ProjT, FWD_PLAIN, R>; break;
    case FWD_MLEM: fn = (const void *)fwd_slab_kernel<VolT, ProjT, FWD_MLEM, R>; break;
    case FWD_SART: fn = (const void *)fwd_slab_kernel<VolT, ProjT, FWD_SART, R>; break;
    case FWD_RESID: fn = (const void *)fwd_slab_kernel<VolT, ProjT, FWD_RESID, R>; break;
    }
    KV_CHECK_CUDA(plan->ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    LaunchTimer lt(plan->ctx, "exact_fwd");
    switch (mode) {
    case FWD_PLAIN: fwd_slab_kernel<VolT, ProjT, FWD_PLAIN, R><<<grid, kThreads, smem, st>>>(map, G, t, a, partials, A); break;
    case FWD_MLEM: fwd_slab_kernel<VolT, ProjT, FWD_MLEM, R><<<grid, kThreads, smem, st>>>(map, G, t, a, partials, A); break;
    case FWD_SART: fwd_slab_kernel<VolT, ProjT, FWD_SART, R><<<grid, kThreads, smem, st>>>(map, G, t, a, partials, A); break;
    case FWD_RESID: fwd_slab_kernel<VolT, ProjT, FWD_RESID, R><<<grid, kThreads, smem, st>>>(map, G, t, a, partials, A); break;
    }
    KV_CHECK_LAUNCH(plan->ctx, "fwd_slab_kernel");
    return KV_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

bool fwd_slab_fit(const kv_plan *plan, int R, int S, int stages, int group, FwdSlabCfg *out, std::string *why) {
    const kv_geometry &g = plan->g;
    const ExactHostTables &H = plan->hx;
    const int es = (int)kv_storage_bytes(plan->storage);
    const int align = 16 / es;
    auto no = [&](const char *m) {
        if (why) *why = m;
        return false;
    };
    if (R != 2 && R != 4 && R != 8) return no("rays per thread must be 2, 4 or 8");
    if (S < 1 || S > 8 || S * 8 * R > kThreads) return no("slab depth out of range");
    if (stages < 2 || stages > kMaxStages) return no("stage count out of range");
    if (group < 1) return no("view group must be positive");
    if (kvtma::encoder() == nullptr) return no("cuTensorMapEncodeTiled is not available");
    if (((size_t)g.nx * es) % 16 != 0) return no("volume rows are not a whole number of 16-byte units");
    if (H.xt.size() != (size_t)g.n_views * g.nu || H.yt.size() != (size_t)g.n_views * g.nv)
        return no("host tables missing");
    for (const float4 &x : H.xt)
        if (!(std::fabs(x.z) >= 0.5f)) return no("a ray crosses more than two voxel-column planes within one slice");
    for (const float4 &y : H.yt)
        if (!(std::fabs(y.z) >= 0.25f)) return no("a ray crosses more than four voxel-row planes within one slice");
    const int TV = 8 * R;
    const int n_ut = (g.nu + 31) / 32, n_vt = (g.nv + TV - 1) / TV;
    const int nslab = (g.nz + S - 1) / S;
    if ((long long)n_ut * n_vt * g.n_views >= (1ll << 31)) return no("grid too large");
    int bx = 0, by = 0;
    const float4 Z{0.f, 0.f, 0.f, 0.f};
    for (int p = 0; p < g.n_views; ++p) {
        const float *hr = H.hr.data() + (size_t)p * (g.nz + 1);
        for (int s = 0; s < nslab; ++s) {
            const float h0 = hr[s * S], h1 = hr[std::min(s * S + S, g.nz)];
            for (int ut = 0; ut < n_ut; ++ut) {
                const size_t a0 = (size_t)p * g.nu + ut * 32, a1 = (size_t)p * g.nu + std::min(ut * 32 + 31, g.nu - 1);
                int x0, y0, nx_, ny_;
                box_origin(H.xt[a0], H.xi[a0], H.xt[a1], H.xi[a1], Z, 0, Z, 0, h0, h1, align, x0, y0, nx_, ny_);
                bx = std::max(bx, nx_);
            }
            for (int vt = 0; vt < n_vt; ++vt) {
                const size_t b0 = (size_t)p * g.nv + vt * TV, b1 = (size_t)p * g.nv + std::min(vt * TV + TV - 1, g.nv - 1);
                int x0, y0, nx_, ny_;
                box_origin(Z, 0, Z, 0, H.yt[b0], H.yi[b0], H.yt[b1], H.yi[b1], h0, h1, align, x0, y0, nx_, ny_);
                by = std::max(by, ny_);
            }
        }
    }
    bx = (bx + align - 1) / align * align;
    if (bx > 256 || by > 256) return no("the rays of one tile spread over more than 256 voxels in a slab");
    const SmemLayout L = smem_layout(R, S, stages, bx, by, g.nz, es);
    if (L.total > 200 * 1024) return no("slab stages do not fit in shared memory");
    FwdSlabCfg c;
    c.R = R;
    c.S = S;
    c.stages = stages;
    c.group = std::min(group, g.n_views);
    c.BX = bx;
    c.BY = by;
    c.smem = L.total;
    *out = c;
    return true;
}

int fwd_slab_default_group(int n_views) {
    const int groups = (n_views + 15) / 16;
    return (n_views + groups - 1) / groups;
}

size_t fwd_slab_blocks(const kv_plan *plan, int n_views) {
    const FwdSlabCfg &c = plan->fslab;
    const int TV = 8 * c.R;
    return (size_t)((plan->g.nu + 31) / 32) * ((plan->g.nv + TV - 1) / TV) * n_views;
}

kv_status fwd_slab_launch(kv_plan *plan, const ExactTables &t, int P, FwdMode mode, const FwdArgs &a,
                          double *partials) {
    const FwdSlabCfg &c = plan->fslab;
    const kv_geometry &g = plan->g;
    const int es = (int)kv_storage_bytes(plan->storage);
    if (reinterpret_cast<uintptr_t>(a.vol) % 16 != 0)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "volume buffer is not 16-byte aligned");
    CUtensorMap map;
    const CUtensorMapDataType dt = plan->storage == KV_STORAGE_BF16  ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                   : plan->storage == KV_STORAGE_F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                     : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)g.nx * es, (cuuint64_t)g.nx * g.ny * es};
    cuuint32_t box[3] = {(cuuint32_t)c.BX, (cuuint32_t)c.BY, (cuuint32_t)c.S};
    cuuint32_t estr[3] = {1, 1, 1};
    if (kvtma::encoder()(&map, dt, 3, const_cast<void *>(a.vol), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return kv_fail(plan->ctx, KV_ERR_CUDA, "volume tensor map rejected");
    const SmemLayout L = smem_layout(c.R, c.S, c.stages, c.BX, c.BY, g.nz, es);
    SlabArgs A;
    A.S = c.S;
    A.BX = c.BX;
    A.BY = c.BY;
    A.stages = c.stages;
    A.nslab = (g.nz + c.S - 1) / c.S;
    A.group = std::min(c.group, P);
    A.n_ut = (g.nu + 31) / 32;
    A.n_vt = (g.nv + 8 * c.R - 1) / (8 * c.R);
    A.align = 16 / es;
    A.stage_elems = L.stage_stride / es;
    A.stage_bytes = (uint32_t)c.BX * c.BY * c.S * es;
    A.desc_off = L.desc_off;
    A.hr_off = L.hr_off;
    A.yt_off = L.yt_off;
    A.yi_off = L.yi_off;
    A.org_off = L.org_off;
    A.status = plan->ctx->d_status;
    const ExGeom G{g.nx, g.ny, g.nz, g.nu, g.nv, P};
    const unsigned grid = (unsigned)((size_t)A.n_ut * A.n_vt * P);
    switch (plan->storage) {
    case KV_STORAGE_BF16:
        if (c.R == 8) return slab_launch_r<__nv_bfloat16, __nv_bfloat16, 8>(plan, map, G, t, mode, a, partials, A, grid, L.total);
        return c.R == 4 ? slab_launch_r<__nv_bfloat16, __nv_bfloat16, 4>(plan, map, G, t, mode, a, partials, A, grid, L.total)
                        : slab_launch_r<__nv_bfloat16, __nv_bfloat16, 2>(plan, map, G, t, mode, a, partials, A, grid, L.total);
    case KV_STORAGE_F16:
        if (c.R == 8) return slab_launch_r<__half, __half, 8>(plan, map, G, t, mode, a, partials, A, grid, L.total);
        return c.R == 4 ? slab_launch_r<__half, __half, 4>(plan, map, G, t, mode, a, partials, A, grid, L.total)
                        : slab_launch_r<__half, __half, 2>(plan, map, G, t, mode, a, partials, A, grid, L.total);
    default:
        if (c.R == 8) return slab_launch_r<float, float, 8>(plan, map, G, t, mode, a, partials, A, grid, L.total);
        return c.R == 4 ? slab_launch_r<float, float, 4>(plan, map, G, t, mode, a, partials, A, grid, L.total)
                        : slab_launch_r<float, float, 2>(plan, map, G, t, mode, a, partials, A, grid, L.total);
    }
}
