// kv_exact.cu -- EXACT family: Siddon line-integral projector A and its exact
// transpose A^T for the linear-sweep tomosynthesis geometry, on sm_103a.
//
// Geometry of a ray.  The detector plane is horizontal, below the volume, and
// every source is above it.  The x coordinate of the ray through detector
// pixel (u,v) at height z depends only on u (and the view), its y coordinate
// only on v.  Every ray crosses every z-plane, so the volume is traversed one
// z-slice at a time with a slice-local parameter t in [0,1] (t = 0 on the
// slice's top plane, t = 1 on its bottom plane).  The length of the ray inside
// voxel (i,j,k) is
//     Ls(u,v) * [min(1, tx_hi(u,i,k), ty_hi(v,j,k)) - max(0, tx_lo, ty_lo)]+
// where [tx_lo, tx_hi] is the t-interval in which ray column u lies in the
// x-slab of column i inside slice k (likewise for y) and Ls = |ray| * dz / H
// the length of the ray within one slice.
//
// The forward kernel walks each ray through its voxels (incremental Siddon:
// R. L. Siddon, Med. Phys. 12(2) 1985; F. Jacobs et al. 1998) and the
// backprojector gathers, for each voxel, the rays crossing it.  Both evaluate
// the plane-crossing parameters with the same float expression
// (cross_t) from the same per-view tables, so every weight the backprojector
// uses is bit-identical to the one the forward projector uses: A^T is the
// exact transpose of A up to the order of the sums.
#include "kv_internal.h"
#include "kv_exact_common.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

namespace {

// Range [k0, k1] of slices in which the ray may be inside the volume laterally.
__device__ __forceinline__ void lateral_slices(float pos0, float slope, int n, int nz, float &klo,
                                               float &khi) {
    // pos(k) = pos0 + slope * k must stay in [0, n]
    if (fabsf(slope) < 1e-30f) {
        if (pos0 < 0.f || pos0 > (float)n) { klo = 1.f; khi = 0.f; }
        else { klo = 0.f; khi = (float)nz; }
        return;
    }
    float a = (0.f - pos0) / slope, b = ((float)n - pos0) / slope;
    klo = fminf(a, b);
    khi = fmaxf(a, b);
}

// One tile of 32 x blockDim.y rays of view p (tile coordinates bx, by) --
// the body of the forward kernel, shared by the per-plan launch and the
// batched persistent kernel.  blin: linear tile index for the partial sums.
template <typename VolT, typename ProjT, int MODE>
__device__ __forceinline__ void fwd_tile(const ExGeom &G, const ExactTables &T, const FwdArgs &a,
                                         double *partials, int bx, int by, int p, size_t blin) {
    const int u = bx * 32 + threadIdx.x;
    const int v = by * blockDim.y + threadIdx.y;
    const bool live = (u < G.nu) && (v < G.nv);
    float acc = 0.f, wsum = 0.f, q = 0.f, pm = 0.f;
    size_t ray = 0;
    if (live) {
        const float4 X = T.xt[(size_t)p * G.nu + u];
        const int ib = T.xi[(size_t)p * G.nu + u];
        const float4 Y = T.yt[(size_t)p * G.nv + v];
        const int jb = T.yi[(size_t)p * G.nv + v];
        const float4 VI = T.vinfo[p];
        const float *hr = T.hr + (size_t)p * (G.nz + 1);
        const int mvx = X.z > 0.f ? 1 : -1, mvy = Y.z > 0.f ? 1 : -1;
        const int ex = mvx > 0 ? 1 : 0, ey = mvy > 0 ? 1 : 0;

        // lateral clipping to the slices the ray can reach inside the volume
        const float hr0 = hr[0], dh = VI.y;
        float kxl, kxh, kyl, kyh;
        lateral_slices((float)ib + fmaf(X.y, hr0, X.x), X.y * dh, G.nx, G.nz, kxl, kxh);
        lateral_slices((float)jb + fmaf(Y.y, hr0, Y.x), Y.y * dh, G.ny, G.nz, kyl, kyh);
        // clamp in float first: converting a huge value saturates and the -1 / +1 would wrap
        const float klo = fmaxf(fmaxf(kxl, kyl), -2.f), khi = fminf(fminf(kxh, kyh), (float)G.nz + 2.f);
        int k0 = 0, k1 = -1;
        if (klo <= khi) {
            k0 = max(0, (int)floorf(klo) - 1);
            k1 = min(G.nz - 1, (int)ceilf(khi) + 1);
        }
        // interior slices: the whole path in the slice stays two voxels away
        // from the lateral faces, so no voxel it visits needs a bounds check
        float ixl, ixh, iyl, iyh;
        lateral_slices((float)ib + fmaf(X.y, hr0, X.x) - 2.f, X.y * dh, G.nx - 4, G.nz, ixl, ixh);
        lateral_slices((float)jb + fmaf(Y.y, hr0, Y.x) - 2.f, Y.y * dh, G.ny - 4, G.nz, iyl, iyh);
        const float kil = fmaxf(fmaxf(ixl, iyl), -2.f), kih = fminf(fminf(ixh, iyh), (float)G.nz + 2.f);
        int ki0 = (int)ceilf(kil), ki1 = (int)floorf(kih) - 1;   // slice k needs planes k, k+1 inside
        if (G.nx < 5 || G.ny < 5) {   // no interior: the margins above would invert
            ki0 = 1;
            ki1 = 0;
        }

        const VolT *vol = static_cast<const VolT *>(a.vol);
        const size_t plane = (size_t)G.nx * G.ny;
        const float fmvx = (float)mvx, fmvy = (float)mvy;
        const int step_y = mvy * G.nx;
        for (int k = k1; k >= k0; --k) {
            const float htop = hr[k + 1];
            const float ftx = __fmaf_rn(X.y, htop, X.x);
            const float fty = __fmaf_rn(Y.y, htop, Y.x);
            const int i = mvx > 0 ? (int)floorf(ftx) : (int)ceilf(ftx) - 1;
            const int j = mvy > 0 ? (int)floorf(fty) : (int)ceilf(fty) - 1;
            // next x / y plane as floats (exact integers): cross_t without conversions
            float fxp = (float)(i + ex), fyp = (float)(j + ey);
            float tx = __fmul_rn(__fsub_rn(fxp, ftx), X.z);
            float ty = __fmul_rn(__fsub_rn(fyp, fty), Y.z);
            float t = 0.f;
            const VolT *slice = vol + (size_t)k * plane;
            if (k >= ki0 && k <= ki1) {
                // Row segments of the (warp-uniform) y walk; inside each, the
                // lane's x crossings.  Weights: same expressions as the
                // backprojector's min(1, tx_hi, ty_hi) - max(0, tx_lo, ty_lo).
                const VolT *ptr = slice + (size_t)(jb + j) * G.nx + (ib + i);
                while (true) {
                    const float tb = fminf(ty, 1.0f);
                    const bool cross = tx < tb;
                    const float te = fminf(tx, tb);
                    const float w = __fsub_rn(te, t);
                    acc = fmaf(w, Store<VolT>::ld(ptr), acc);
                    if (MODE == FWD_SART) wsum += w;
                    // the common case -- at most one column crossing in the
                    // row segment -- without a divergent branch
                    float vc = cross ? Store<VolT>::ld(ptr + mvx) : 0.f;
                    ptr += cross ? mvx : 0;
                    fxp += cross ? fmvx : 0.f;
                    tx = __fmul_rn(__fsub_rn(fxp, ftx), X.z);
                    float tc = te;
                    while (tx < tb) {   // rarely: a second crossing in the same row
                        const float w2 = __fsub_rn(tx, tc);
                        acc = fmaf(w2, vc, acc);
                        if (MODE == FWD_SART) wsum += w2;
                        tc = tx;
                        ptr += mvx;
                        fxp += fmvx;
                        tx = __fmul_rn(__fsub_rn(fxp, ftx), X.z);
                        vc = Store<VolT>::ld(ptr);
                    }
                    const float w3 = __fsub_rn(tb, tc);
                    acc = fmaf(w3, vc, acc);
                    if (MODE == FWD_SART) wsum += w3;
                    t = tb;
                    if (tb >= 1.0f) break;
                    ptr += step_y;
                    fyp += fmvy;
                    ty = __fmul_rn(__fsub_rn(fyp, fty), Y.z);
                }
            } else {
                int ai = ib + i, aj = jb + j;
                while (true) {
                    const float tb = fminf(ty, 1.0f);
                    const bool row_in = (unsigned)aj < (unsigned)G.ny;
                    const VolT *row = slice + (size_t)(row_in ? aj : 0) * G.nx;
                    while (tx < tb) {
                        if (row_in && (unsigned)ai < (unsigned)G.nx) {
                            const float w = __fsub_rn(tx, t);
                            acc = fmaf(w, Store<VolT>::ld(row + ai), acc);
                            if (MODE == FWD_SART) wsum += w;
                        }
                        t = tx;
                        ai += mvx;
                        fxp += fmvx;
                        tx = __fmul_rn(__fsub_rn(fxp, ftx), X.z);
                    }
                    if (row_in && (unsigned)ai < (unsigned)G.nx) {
                        const float w = __fsub_rn(tb, t);
                        acc = fmaf(w, Store<VolT>::ld(row + ai), acc);
                        if (MODE == FWD_SART) wsum += w;
                    }
                    t = tb;
                    if (tb >= 1.0f) break;
                    aj += mvy;
                    fyp += fmvy;
                    ty = __fmul_rn(__fsub_rn(fyp, fty), Y.z);
                }
            }
        }
        const float ls = ray_factor(X.w, Y.w, VI);
        q = acc * ls;
        ray = ((size_t)p * G.nv + v) * G.nu + u;
        ProjT *out = static_cast<ProjT *>(a.out);
        if (MODE != FWD_PLAIN) pm = Store<ProjT>::ld(static_cast<const ProjT *>(a.meas) + ray);
        if (MODE == FWD_PLAIN) {
            Store<ProjT>::st(out + ray, q);
        } else if (MODE == FWD_MLEM) {
            const float r = q > 0.f ? a.relax * pm / q : 0.f;
            Store<ProjT>::st(out + ray, r * ls);
        } else if (MODE == FWD_SART) {
            const float rows = wsum * ls;
            const float r = rows > 0.f ? (pm - q) / rows : 0.f;
            Store<ProjT>::st(out + ray, r * ls);
        }
    }
    if (partials != nullptr) {
        // FP64 block reduction of (q - p)^2, p^2 and p log q - q
        double d0 = 0.0, d1 = 0.0, d2 = 0.0;
        if (live) {
            const double dq = (double)q - (double)pm;
            d0 = dq * dq;
            d1 = (double)pm * (double)pm;
            d2 = (q > 0.f ? (double)pm * (double)logf(q) : 0.0) - (double)q;
        }
        for (int o = 16; o > 0; o >>= 1) {
            d0 += __shfl_xor_sync(0xffffffffu, d0, o);
            d1 += __shfl_xor_sync(0xffffffffu, d1, o);
            d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        }
        __shared__ double red[3][32];
        const int warp = threadIdx.y, nwarps = blockDim.y;
        if (threadIdx.x == 0) { red[0][warp] = d0; red[1][warp] = d1; red[2][warp] = d2; }
        __syncthreads();
        if (warp == 0) {
            d0 = threadIdx.x < nwarps ? red[0][threadIdx.x] : 0.0;
            d1 = threadIdx.x < nwarps ? red[1][threadIdx.x] : 0.0;
            d2 = threadIdx.x < nwarps ? red[2][threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) {
                d0 += __shfl_xor_sync(0xffffffffu, d0, o);
                d1 += __shfl_xor_sync(0xffffffffu, d1, o);
                d2 += __shfl_xor_sync(0xffffffffu, d2, o);
            }
            if (threadIdx.x == 0) {
                partials[3 * blin + 0] = d0;
                partials[3 * blin + 1] = d1;
                partials[3 * blin + 2] = d2;
            }
        }
    }
}

template <typename VolT, typename ProjT, int MODE>
__global__ void __launch_bounds__(256) exact_fwd_kernel(ExGeom G, ExactTables T, FwdArgs a,
                                                        double *partials) {
    fwd_tile<VolT, ProjT, MODE>(G, T, a, partials, blockIdx.x, blockIdx.y, blockIdx.z,
                                ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
}

// Sums the per-block partials into out[0..2] (single block).
__global__ void reduce_partials_kernel(const double *partials, size_t nblocks, double *out) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (size_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
        s0 += partials[3 * b];
        s1 += partials[3 * b + 1];
        s2 += partials[3 * b + 2];
    }
    __shared__ double sh[3][1024];
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
    if (threadIdx.x == 0) {
        out[0] = sh[0][0];
        out[1] = sh[1][0];
        out[2] = sh[2][0];
    }
}

// y'(u,v) = y(u,v) * Ls(u,v)   (y == nullptr: y' = Ls, used for A^T 1)
template <typename ProjT>
__global__ void prescale_kernel(ExGeom G, ExactTables T, const float *y, ProjT *yp) {
    const int u = blockIdx.x * 32 + threadIdx.x;
    const int v = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (u >= G.nu || v >= G.nv) return;
    const float ls = ray_factor(T.xt[(size_t)p * G.nu + u].w, T.yt[(size_t)p * G.nv + v].w, T.vinfo[p]);
    const size_t r = ((size_t)p * G.nv + v) * G.nu + u;
    Store<ProjT>::st(yp + r, y ? y[r] * ls : ls);
}

// Gather backprojector.  Block = 32 x BY voxels (i fastest) of one slice k;
// warp w owns row j.  For every view, each warp computes the slice-local
// y-intervals of its candidate detector rows once into shared memory; each
// lane holds the x-intervals of its voxel's candidate detector columns in
// registers (up to BACK_SLOTS at a time) and accumulates over (candidate row,
// candidate column), in a row loop unrolled for the warp's slot count.
// (Computing the x-intervals once per block in shared memory instead -- they
// depend on the column, not the row -- measured slower: the two block
// barriers per view cost more than the redundant interval arithmetic.)
// Accumulators of the backprojector: plain FP32 (every storage mode: with
// 16-bit ratio images and volumes, their rounding dominates; a compensated
// sum measured the same errors to three digits after 50 MLEM iterations and
// cost a quarter of the iteration), and a double-float sum of exact products
// (TwoProduct + TwoSum in FP32 arithmetic, ~1e-14 relative) for the FP64
// sensitivity image.
enum { ACC_F32 = 0, ACC_DF = 2 };

// Candidate detector columns a lane holds in registers at once (a voxel at
// the chest-DT geometry has 4-7).
constexpr int BACK_SLOTS = 8;

// One backprojection term w * y into the accumulator (acc, comp).
template <int ACC>
__device__ __forceinline__ void back_accumulate(float w, float yv, float &acc, float &comp) {
    if (ACC == ACC_DF) {            // exact product + TwoSum: a double-float sum
        const float pr = __fmul_rn(w, yv);
        const float pe = __fmaf_rn(w, yv, -pr);
        const float s_ = __fadd_rn(acc, pr);
        const float bp = __fsub_rn(s_, acc);
        const float er = __fadd_rn(__fsub_rn(acc, __fsub_rn(s_, bp)), __fsub_rn(pr, bp));
        acc = s_;
        comp = __fadd_rn(comp, __fadd_rn(er, pe));
    } else {
        acc = fmaf(w, yv, acc);
    }
}

// The (candidate row, candidate column) terms of one voxel: nvc rows of
// y-intervals ys[] against NS column slots of x-intervals in registers.
template <int NS, typename ProjT, int ACC>
__device__ __forceinline__ void back_rows(const ProjT *row, int nu, int nvc, const float2 *ys,
                                          const float (&lox)[BACK_SLOTS], const float (&hix)[BACK_SLOTS],
                                          float &acc, float &comp) {
    for (int c = 0; c < nvc; ++c, row += nu) {
        const float2 yi = ys[c];
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const float w = __fsub_rn(fminf(hix[s], yi.y), fmaxf(lox[s], yi.x));
            if (w > 0.f) back_accumulate<ACC>(w, Store<ProjT>::ld(row + s), acc, comp);
        }
    }
}

template <typename VolT, typename ProjT, int ACC, int MODE>
__device__ __forceinline__ void back_tile(const ExGeom &G, const ExactTables &T, const BackArgs &a,
                                          double *sens_out, int bx, int by, int k) {
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int i = bx * 32 + lane;
    const int j = by * blockDim.y + warp;
    __shared__ float2 ysh[16][32];
    const bool live_i = i < G.nx;
    const bool live_j = j < G.ny;   // warp-uniform
    const ProjT *yp = static_cast<const ProjT *>(a.yp);
    float acc = 0.f, comp = 0.f;
    if (live_j) {
        for (int p = 0; p < G.n_views; ++p) {
            const float *hr = T.hr + (size_t)p * (G.nz + 1);
            const float htop = hr[k + 1];
            const float4 r0 = T.rng[(size_t)p * (G.nz + 1) + k];
            const float4 r1 = T.rng[(size_t)p * (G.nz + 1) + k + 1];
            // candidate detector rows of voxel row j (warp-uniform)
            const float vlo = fminf(((float)j - r0.z) * r0.w, ((float)j - r1.z) * r1.w);
            const float vhi = fmaxf(((float)(j + 1) - r0.z) * r0.w, ((float)(j + 1) - r1.z) * r1.w);
            const int v0 = max(0, (int)ceilf(fminf(vlo, vhi) - 0.01f));
            const int v1 = min(G.nv - 1, (int)floorf(fmaxf(vlo, vhi) + 0.01f));
            // candidate detector columns of voxel column i (per lane)
            const float ulo = fminf(((float)i - r0.x) * r0.y, ((float)i - r1.x) * r1.y);
            const float uhi = fmaxf(((float)(i + 1) - r0.x) * r0.y, ((float)(i + 1) - r1.x) * r1.y);
            int u0 = max(0, (int)ceilf(fminf(ulo, uhi) - 0.01f));
            int u1 = min(G.nu - 1, (int)floorf(fmaxf(ulo, uhi) + 0.01f));
            if (!live_i) u1 = u0 - 1;
            for (int vb = v0; vb <= v1; vb += 32) {
                const int vv = vb + lane;
                if (vv <= v1) {
                    const float4 Y = T.yt[(size_t)p * G.nv + vv];
                    const int jb = T.yi[(size_t)p * G.nv + vv];
                    const float fty = __fmaf_rn(Y.y, htop, Y.x);
                    const float ta = cross_t(j - jb, fty, Y.z), tb = cross_t(j + 1 - jb, fty, Y.z);
                    ysh[warp][lane] = make_float2(fmaxf(0.f, fminf(ta, tb)), fminf(1.f, fmaxf(ta, tb)));
                }
                __syncwarp();
                const int nvc = min(32, v1 - vb + 1);
                // the lane's candidate columns, up to BACK_SLOTS at a time, with
                // their x-intervals in registers; empty slots get lo > hi.
                // The chunk loop runs the same number of times in every lane
                // (the widest lane's count, taken while the warp is converged),
                // so slots beyond it are skipped with a warp-uniform branch.
                const int n_u = u1 >= u0 ? u1 - u0 + 1 : 0;
                const int n_u_warp = __reduce_max_sync(0xffffffffu, n_u);
                for (int cb = 0; cb * BACK_SLOTS < n_u_warp; ++cb) {
                    const int ub = u0 + cb * BACK_SLOTS;
                    const int nslot = min(BACK_SLOTS, n_u_warp - cb * BACK_SLOTS);
                    float lox[BACK_SLOTS], hix[BACK_SLOTS];
#pragma unroll
                    for (int s = 0; s < BACK_SLOTS; ++s) {
                        lox[s] = 1.f;
                        hix[s] = 0.f;
                        const int u = ub + s;
                        if (u <= u1) {
                            const float4 X = T.xt[(size_t)p * G.nu + u];
                            const int ib = T.xi[(size_t)p * G.nu + u];
                            const float ftx = __fmaf_rn(X.y, htop, X.x);
                            const float ta = cross_t(i - ib, ftx, X.z), tb = cross_t(i + 1 - ib, ftx, X.z);
                            lox[s] = fmaxf(0.f, fminf(ta, tb));
                            hix[s] = fminf(1.f, fmaxf(ta, tb));
                        }
                    }
                    const ProjT *row = yp + ((size_t)p * G.nv + vb) * G.nu + ub;
                    // nslot is warp-uniform: one unrolled row loop per slot count
                    switch (nslot) {
                    case 1: back_rows<1, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    case 2: back_rows<2, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    case 3: back_rows<3, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    case 4: back_rows<4, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    case 5: back_rows<5, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    case 6: back_rows<6, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    case 7: back_rows<7, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    default: back_rows<8, ProjT, ACC>(row, G.nu, nvc, ysh[warp], lox, hix, acc, comp); break;
                    }
                }
                __syncwarp();
            }
        }
    }
    if (!live_i || !live_j) return;
    const size_t idx = ((size_t)k * G.ny + j) * G.nx + i;
    if (sens_out != nullptr) {
        sens_out[idx] = ACC == ACC_DF ? (double)acc + (double)comp : (double)acc;
        return;
    }
    VolT *vol = static_cast<VolT *>(a.vol);
    const float b = (float)acc;
    if (MODE == BACK_PLAIN) {
        Store<VolT>::st(vol + idx, b);
    } else if (MODE == BACK_MLEM) {
        const double s = a.sens[idx];
        if (s > 0.0) Store<VolT>::st(vol + idx, (float)((double)Store<VolT>::ld_rw(vol + idx) * (double)b / s));
    } else if (MODE == BACK_SART) {
        const double s = a.sens[idx];
        if (s > 0.0)
            Store<VolT>::st(vol + idx, Store<VolT>::ld_rw(vol + idx) + (float)((double)(a.relax * b) / s));
    }
}

template <typename VolT, typename ProjT, int ACC, int MODE>
__global__ void __launch_bounds__(256) exact_back_kernel(ExGeom G, ExactTables T, BackArgs a,
                                                         double *sens_out, int z0) {
    // slices z0 .. z0 + gridDim.z - 1 (z0 = 0 and gridDim.z = nz for the whole volume)
    back_tile<VolT, ProjT, ACC, MODE>(G, T, a, sens_out, blockIdx.x, blockIdx.y, z0 + (int)blockIdx.z);
}

// ---------------------------------------------------------------------------
// Gather backprojector, R voxel rows and S slices per thread.  Block = 32 x 8
// threads over 32 voxel columns (lanes) by 8R voxel rows (warp w owns rows
// w, w + 8, ...) and S consecutive slices; views are the outer loop, so the
// S slices read nearly the same detector patch of a view while it sits in
// L1.  For each (view, slice) a lane computes the x-intervals of its voxel
// column's candidate detector columns once -- only as many slots as the
// warp's widest voxel needs -- and uses them for its R voxel rows; the
// candidate detector rows of the R voxel rows go to shared memory as
// t-intervals, computed side by side (lane group q of 32/R lanes evaluates
// row q's range and intervals, one lane per candidate, so a warp fills all R
// rows in one pass when each has at most 32/R candidates); the pairs are
// visited in the same order for every R.  The R voxel rows then run through
// their candidate rows in lockstep (independent accumulators, so their loads
// and sums overlap).  Weights are the same float expressions as back_tile's,
// bit for bit.
// ---------------------------------------------------------------------------

// The terms of one chunk of NS candidate columns (ub .. ub + NS - 1) for the
// R voxels of this thread, candidate rows c < nvc of the current row chunk.
template <int NS, int R, typename ProjT, int ACC>
__device__ __forceinline__ void back_chunk_r(const ExGeom &G, const ExactTables &T, int p, float htop, int i,
                                             int ub, int u1, const ProjT *const (&rowp)[R], int nvc,
                                             const float2 (*ys)[32], float *acc, float *comp) {
    float lox[NS], hix[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        lox[s] = 1.f;
        hix[s] = 0.f;
        const int u = ub + s;
        if (u <= u1) {
            const float4 X = T.xt[(size_t)p * G.nu + u];
            const int ib = T.xi[(size_t)p * G.nu + u];
            const float ftx = __fmaf_rn(X.y, htop, X.x);
            // the two bounding planes as exact float integers (one conversion)
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
            const ProjT *row = rowp[q] + (size_t)c * G.nu;
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                const float w = __fsub_rn(fminf(hix[s], yi.y), fmaxf(lox[s], yi.x));
                if (w > 0.f) back_accumulate<ACC>(w, Store<ProjT>::ld(row + s), acc[q], comp[q]);
            }
        }
    }
}

template <typename VolT, typename ProjT, int ACC, int R, int S>
__device__ __forceinline__ void back_tile_r(const ExGeom &G, const ExactTables &T, const BackArgs &a,
                                            double *sens_out, int bx, int by, int k0, int kend, int mode) {
    constexpr int CW = 32 / R;                 // candidates of one voxel row filled per pass
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int i = bx * 32 + lane;
    const int jw = by * 8 * R + warp;          // voxel row of q = 0; rows jw + 8q
    const int qf = lane / CW, cf = lane % CW;  // this lane fills candidate cf (+ CW f) of row qf
    const int jf = jw + 8 * qf;
    __shared__ float2 ysh[8][R][32];
    const bool live_i = i < G.nx;
    const ProjT *yp = static_cast<const ProjT *>(a.yp);
    float acc[S][R], comp[S][R];
#pragma unroll
    for (int kk = 0; kk < S; ++kk)
#pragma unroll
        for (int q = 0; q < R; ++q) acc[kk][q] = comp[kk][q] = 0.f;
    for (int p = 0; p < G.n_views; ++p) {
#pragma unroll
        for (int kk = 0; kk < S; ++kk) {
            const int k = k0 + kk;
            if (k >= kend) break;   // block-uniform
            const float htop = T.hr[(size_t)p * (G.nz + 1) + k + 1];
            const float4 r0 = T.rng[(size_t)p * (G.nz + 1) + k];
            const float4 r1 = T.rng[(size_t)p * (G.nz + 1) + k + 1];
            // candidate detector columns of voxel column i (per lane)
            const float ulo = fminf(((float)i - r0.x) * r0.y, ((float)i - r1.x) * r1.y);
            const float uhi = fmaxf(((float)(i + 1) - r0.x) * r0.y, ((float)(i + 1) - r1.x) * r1.y);
            const int u0 = max(0, (int)ceilf(fminf(ulo, uhi) - 0.01f));
            int u1 = min(G.nu - 1, (int)floorf(fmaxf(ulo, uhi) + 0.01f));
            if (!live_i) u1 = u0 - 1;
            const int n_u_warp = __reduce_max_sync(0xffffffffu, u1 >= u0 ? u1 - u0 + 1 : 0);
            // candidate detector rows of the lane's fill row: the R rows are
            // evaluated side by side in lane groups of CW, and each row's first
            // candidate is broadcast from the first lane of its group
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
                // the rows' candidate intervals, CW candidates of each row per pass;
                // entries past a row's candidates are empty (lo > hi) and weigh nothing
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
                for (int cb = 0; cb * BACK_SLOTS < n_u_warp; ++cb) {
                    const int ub = u0 + cb * BACK_SLOTS;
                    const int nslot = min(BACK_SLOTS, n_u_warp - cb * BACK_SLOTS);
                    const ProjT *rowp[R];
#pragma unroll
                    for (int q = 0; q < R; ++q) rowp[q] = yp + ((size_t)p * G.nv + v0[q] + vb) * G.nu + ub;
                    float *ak = acc[kk], *ck = comp[kk];
                    // nslot is warp-uniform: one unrolled chunk per slot count
                    switch (nslot) {
                    case 1: back_chunk_r<1, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    case 2: back_chunk_r<2, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    case 3: back_chunk_r<3, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    case 4: back_chunk_r<4, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    case 5: back_chunk_r<5, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    case 6: back_chunk_r<6, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    case 7: back_chunk_r<7, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    default: back_chunk_r<8, R, ProjT, ACC>(G, T, p, htop, i, ub, u1, rowp, nvc, ysh[warp], ak, ck); break;
                    }
                }
                __syncwarp();
            }
        }
    }
    if (!live_i) return;
#pragma unroll
    for (int kk = 0; kk < S; ++kk) {
        const int k = k0 + kk;
        if (k >= kend) break;
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int j = jw + 8 * q;
            if (j >= G.ny) continue;
            const size_t idx = ((size_t)k * G.ny + j) * G.nx + i;
            if (sens_out != nullptr) {
                sens_out[idx] = ACC == ACC_DF ? (double)acc[kk][q] + (double)comp[kk][q] : (double)acc[kk][q];
                continue;
            }
            VolT *vol = static_cast<VolT *>(a.vol);
            const float b = (float)acc[kk][q];
            if (mode == BACK_PLAIN) {
                Store<VolT>::st(vol + idx, b);
            } else if (mode == BACK_MLEM) {
                const double sv = a.sens[idx];
                if (sv > 0.0)
                    Store<VolT>::st(vol + idx, (float)((double)Store<VolT>::ld_rw(vol + idx) * (double)b / sv));
            } else if (mode == BACK_SART) {
                const double sv = a.sens[idx];
                if (sv > 0.0)
                    Store<VolT>::st(vol + idx, Store<VolT>::ld_rw(vol + idx) + (float)((double)(a.relax * b) / sv));
            }
        }
    }
}

// Slices z0 .. z0 + nzs - 1, S per block.  Grid (slice groups, voxel-row
// tiles, voxel-column tiles): the slice group varies fastest, so the blocks
// in flight cover a strip of voxel columns at every height, whose detector
// footprint over all views stays in L2 while the strip's rows are swept
// (slice groups slowest re-read every projection image once per group).
// The pass (plain, MLEM update, SART update) only changes the epilogue: a
// kernel argument, not a template parameter.
template <typename VolT, typename ProjT, int ACC, int R, int S>
__global__ void __launch_bounds__(256) exact_back_r_kernel(ExGeom G, ExactTables T, BackArgs a,
                                                           double *sens_out, int z0, int nzs, int mode) {
    back_tile_r<VolT, ProjT, ACC, R, S>(G, T, a, sens_out, blockIdx.z, blockIdx.y, z0 + S * (int)blockIdx.x,
                                        z0 + nzs, mode);
}

ExGeom exgeom(const kv_plan *plan, int n_views) {
    return ExGeom{plan->g.nx, plan->g.ny, plan->g.nz, plan->g.nu, plan->g.nv, n_views};
}

}  // namespace

// ---------------------------------------------------------------------------
// Tables (host, double precision)
// ---------------------------------------------------------------------------

void exact_free_tables(ExactTables *t) {
    cudaFree(t->xt);
    cudaFree(t->xi);
    cudaFree(t->yt);
    cudaFree(t->yi);
    cudaFree(t->hr);
    cudaFree(t->vinfo);
    cudaFree(t->rng);
    *t = ExactTables{};
}

kv_status exact_build_tables(kv_plan *plan, const float *src, const float *det, int P,
                             ExactTables *out, ExactHostTables *host) {
    const kv_geometry &g = plan->g;
    kv_ctx *ctx = plan->ctx;
    const double X0 = -0.5 * g.nx * (double)g.dx, Y0 = -0.5 * g.ny * (double)g.dy;
    const double Ztop = 0.5 * g.nz * (double)g.dz, Zbot = -Ztop;
    std::vector<float4> xt((size_t)P * g.nu), yt((size_t)P * g.nv), vinfo(P), rng((size_t)P * (g.nz + 1));
    std::vector<int> xi((size_t)P * g.nu), yi((size_t)P * g.nv);
    std::vector<float> hr((size_t)P * (g.nz + 1));
    for (int p = 0; p < P; ++p) {
        const double sx = src[3 * p], sy = src[3 * p + 1], sz = src[3 * p + 2];
        const double ox = det[3 * p], oy = det[3 * p + 1], zd = det[3 * p + 2];
        if (!(sz > Ztop) || !(zd < Zbot))
            return kv_fail(ctx, KV_ERR_GEOMETRY,
                           "view %d: EXACT needs the source above the volume (z=%g > %g) and the "
                           "detector below it (z=%g < %g)", p, sz, Ztop, zd, Zbot);
        const double H = sz - zd, dh = g.dz / H, hmid = -zd / H;
        vinfo[p] = make_float4((float)(H * H), (float)dh, 0.f, 0.f);
        for (int k = 0; k <= g.nz; ++k) {
            const double zk = Zbot + k * (double)g.dz;
            const double h = (zk - zd) / H;
            hr[(size_t)p * (g.nz + 1) + k] = (float)(zk / H);
            // x of column u at plane k: Ax + Bx * u (voxel units)
            const double Bx = g.du * (1.0 - h) / g.dx, By = g.dv * (1.0 - h) / g.dy;
            const double Ax = ((ox - X0) + (sx - ox) * h + 0.5 * g.du * (1.0 - h)) / g.dx;
            const double Ay = ((oy - Y0) + (sy - oy) * h + 0.5 * g.dv * (1.0 - h)) / g.dy;
            rng[(size_t)p * (g.nz + 1) + k] = make_float4((float)Ax, (float)(1.0 / Bx), (float)Ay, (float)(1.0 / By));
        }
        auto axis = [&](int n, double o, double d, double s, double B0, double sp, float4 *tab, int *ib,
                        int &bad) {
            for (int u = 0; u < n; ++u) {
                const double pc = o + (u + 0.5) * d;
                const double c = (pc - B0) / sp;
                double gr = (s - pc) / sp;
                if (std::fabs(gr) < 1e-20) gr = gr < 0 ? -1e-20 : 1e-20;
                if (std::fabs(gr) * dh > 4096.0) bad = 1;  // > 4096 voxel crossings per slice
                const double cm = c + gr * hmid;
                const double base = std::floor(cm);
                tab[u] = make_float4((float)(cm - base), (float)gr, (float)(-1.0 / (gr * dh)), (float)(s - pc));
                ib[u] = (int)base;
            }
        };
        int bad = 0;
        axis(g.nu, ox, g.du, sx, X0, g.dx, xt.data() + (size_t)p * g.nu, xi.data() + (size_t)p * g.nu, bad);
        axis(g.nv, oy, g.dv, sy, Y0, g.dy, yt.data() + (size_t)p * g.nv, yi.data() + (size_t)p * g.nv, bad);
        if (bad)
            return kv_fail(ctx, KV_ERR_GEOMETRY,
                           "view %d: rays cross more than 4096 voxel columns within one slice", p);
    }
    ExactTables t;
    auto up = [&](void **dst, const void *srcp, size_t bytes) -> kv_status {
        KV_CHECK_CUDA(ctx, cudaMalloc(dst, bytes));
        KV_CHECK_CUDA(ctx, cudaMemcpyAsync(*dst, srcp, bytes, cudaMemcpyHostToDevice, ctx->stream));
        return KV_OK;
    };
    kv_status s = KV_OK;
    if ((s = up((void **)&t.xt, xt.data(), xt.size() * sizeof(float4))) != KV_OK ||
        (s = up((void **)&t.xi, xi.data(), xi.size() * sizeof(int))) != KV_OK ||
        (s = up((void **)&t.yt, yt.data(), yt.size() * sizeof(float4))) != KV_OK ||
        (s = up((void **)&t.yi, yi.data(), yi.size() * sizeof(int))) != KV_OK ||
        (s = up((void **)&t.hr, hr.data(), hr.size() * sizeof(float))) != KV_OK ||
        (s = up((void **)&t.vinfo, vinfo.data(), vinfo.size() * sizeof(float4))) != KV_OK ||
        (s = up((void **)&t.rng, rng.data(), rng.size() * sizeof(float4))) != KV_OK) {
        exact_free_tables(&t);
        return s;
    }
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out = t;
    if (host != nullptr) {
        host->xt = std::move(xt);
        host->xi = std::move(xi);
        host->yt = std::move(yt);
        host->yi = std::move(yi);
        host->hr = std::move(hr);
        host->rng = std::move(rng);
    }
    return KV_OK;
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

namespace {
template <typename VolT, typename ProjT>
kv_status fwd_dispatch(kv_plan *plan, const ExactTables &t, int P, FwdMode mode, const FwdArgs &a,
                       double *partials) {
    ExGeom G = exgeom(plan, P);
    dim3 block(32, plan->fwd_by);
    dim3 grid((G.nu + 31) / 32, (G.nv + plan->fwd_by - 1) / plan->fwd_by, P);
    cudaStream_t st = plan->ctx->stream;
    LaunchTimer lt(plan->ctx, "exact_fwd");
    switch (mode) {
    case FWD_PLAIN: exact_fwd_kernel<VolT, ProjT, FWD_PLAIN><<<grid, block, 0, st>>>(G, t, a, partials); break;
    case FWD_MLEM: exact_fwd_kernel<VolT, ProjT, FWD_MLEM><<<grid, block, 0, st>>>(G, t, a, partials); break;
    case FWD_SART: exact_fwd_kernel<VolT, ProjT, FWD_SART><<<grid, block, 0, st>>>(G, t, a, partials); break;
    case FWD_RESID: exact_fwd_kernel<VolT, ProjT, FWD_RESID><<<grid, block, 0, st>>>(G, t, a, partials); break;
    }
    KV_CHECK_LAUNCH(plan->ctx, "exact_fwd_kernel");
    return KV_OK;
}

template <typename VolT, typename ProjT, int ACC, int R, int S>
void back_r_launch(const ExGeom &G, const ExactTables &t, BackMode mode, const BackArgs &a, double *sens_out,
                   int z0, int nzs, cudaStream_t st) {
    dim3 block(32, 8), grid((nzs + S - 1) / S, (G.ny + 8 * R - 1) / (8 * R), (G.nx + 31) / 32);
    exact_back_r_kernel<VolT, ProjT, ACC, R, S><<<grid, block, 0, st>>>(G, t, a, sens_out, z0, nzs, (int)mode);
}

// (rows per thread, slices per thread): (1, 1), (2, 1), (2, 2), (4, 1), (4, 2) or (8, 1)
template <typename VolT, typename ProjT, int ACC>
void back_r_dispatch(int R, int S, const ExGeom &G, const ExactTables &t, BackMode mode, const BackArgs &a,
                     double *sens_out, int z0, int nzs, cudaStream_t st) {
    if (R == 1) back_r_launch<VolT, ProjT, ACC, 1, 1>(G, t, mode, a, sens_out, z0, nzs, st);
    else if (R == 2 && S == 1) back_r_launch<VolT, ProjT, ACC, 2, 1>(G, t, mode, a, sens_out, z0, nzs, st);
    else if (R == 2) back_r_launch<VolT, ProjT, ACC, 2, 2>(G, t, mode, a, sens_out, z0, nzs, st);
    else if (R == 4 && S == 1) back_r_launch<VolT, ProjT, ACC, 4, 1>(G, t, mode, a, sens_out, z0, nzs, st);
    else if (R == 4) back_r_launch<VolT, ProjT, ACC, 4, 2>(G, t, mode, a, sens_out, z0, nzs, st);
    else back_r_launch<VolT, ProjT, ACC, 8, 1>(G, t, mode, a, sens_out, z0, nzs, st);
}

template <typename VolT, typename ProjT>
kv_status back_dispatch(kv_plan *plan, BackMode mode, const BackArgs &a, int z0, int nzs) {
    ExGeom G = exgeom(plan, plan->g.n_views);
    if (std::is_same<VolT, float>::value && plan->bstage.R > 0)
        return back_stage_launch(plan, mode, a, z0, nzs, plan->g.n_views);
    if (plan->back_rows > 0) {
        LaunchTimer lt(plan->ctx, "exact_back");
        back_r_dispatch<VolT, ProjT, ACC_F32>(plan->back_rows, plan->back_slices, G, plan->ex, mode, a, nullptr, z0, nzs, plan->ctx->stream);
        KV_CHECK_LAUNCH(plan->ctx, "exact_back_r_kernel");
        return KV_OK;
    }
    dim3 block(32, plan->back_by);
    dim3 grid((G.nx + 31) / 32, (G.ny + plan->back_by - 1) / plan->back_by, nzs);
    cudaStream_t st = plan->ctx->stream;
    const ExactTables &t = plan->ex;
    LaunchTimer lt(plan->ctx, "exact_back");
    switch (mode) {
    case BACK_PLAIN: exact_back_kernel<VolT, ProjT, ACC_F32, BACK_PLAIN><<<grid, block, 0, st>>>(G, t, a, nullptr, z0); break;
    case BACK_MLEM: exact_back_kernel<VolT, ProjT, ACC_F32, BACK_MLEM><<<grid, block, 0, st>>>(G, t, a, nullptr, z0); break;
    case BACK_SART: exact_back_kernel<VolT, ProjT, ACC_F32, BACK_SART><<<grid, block, 0, st>>>(G, t, a, nullptr, z0); break;
    }
    KV_CHECK_LAUNCH(plan->ctx, "exact_back_kernel");
    return KV_OK;
}
}  // namespace

kv_status exact_forward_launch(kv_plan *plan, const ExactTables &t, int P, FwdMode mode,
                               const FwdArgs &a) {
    if (plan->fwd_by < 1 || plan->fwd_by > 8) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "bad forward block");
    const bool slab = plan->fslab.R > 0;
    double *partials = nullptr;
    size_t nblocks = 0;
    if (a.red != nullptr) {
        nblocks = slab ? fwd_slab_blocks(plan, P)
                       : (size_t)((plan->g.nu + 31) / 32) * ((plan->g.nv + plan->fwd_by - 1) / plan->fwd_by) * P;
        KV_CHECK_CUDA(plan->ctx, cudaMallocAsync((void **)&partials, nblocks * 3 * sizeof(double), plan->ctx->stream));
    }
    kv_status s;
    if (slab) s = fwd_slab_launch(plan, t, P, mode, a, partials);
    else switch (plan->storage) {
    case KV_STORAGE_BF16: s = fwd_dispatch<__nv_bfloat16, __nv_bfloat16>(plan, t, P, mode, a, partials); break;
    case KV_STORAGE_F16: s = fwd_dispatch<__half, __half>(plan, t, P, mode, a, partials); break;
    default: s = fwd_dispatch<float, float>(plan, t, P, mode, a, partials); break;
    }
    if (partials != nullptr) {
        if (s == KV_OK) {
            LaunchTimer lt(plan->ctx, "reduce_partials");
            reduce_partials_kernel<<<1, 1024, 0, plan->ctx->stream>>>(partials, nblocks, a.red);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) s = kv_fail(plan->ctx, KV_ERR_CUDA, "reduce_partials_kernel: %s", cudaGetErrorString(e));
        }
        cudaFreeAsync(partials, plan->ctx->stream);
    }
    return s;
}

// Forward projection of views [v0, v0 + n) only: the per-view tables and the
// projection buffers are offset to view v0, so every ray computes what the
// whole-plan launch computes for it.  No reduction (a.red must be null).
kv_status exact_forward_views_launch(kv_plan *plan, int v0, int n, FwdMode mode, const FwdArgs &a) {
    const kv_geometry &g = plan->g;
    if (v0 < 0 || n < 1 || v0 + n > g.n_views || a.red != nullptr)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "bad view range for the forward projection");
    ExactTables t = plan->ex;
    t.xt += (size_t)v0 * g.nu;
    t.xi += (size_t)v0 * g.nu;
    t.yt += (size_t)v0 * g.nv;
    t.yi += (size_t)v0 * g.nv;
    t.vinfo += v0;
    t.hr += (size_t)v0 * (g.nz + 1);
    t.rng += (size_t)v0 * (g.nz + 1);
    const size_t off = (size_t)v0 * g.nu * g.nv * kv_storage_bytes(plan->storage);
    FwdArgs b = a;
    if (b.meas != nullptr) b.meas = static_cast<const char *>(b.meas) + off;
    b.out = static_cast<char *>(b.out) + off;
    return exact_forward_launch(plan, t, n, mode, b);
}

kv_status exact_back_slab_launch(kv_plan *plan, BackMode mode, const BackArgs &a, int z0, int nzs) {
    if (plan->back_by < 1 || plan->back_by > 8) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "bad back block");
    if (z0 < 0 || nzs < 1 || z0 + nzs > plan->g.nz)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "bad slice range for the backprojection");
    switch (plan->storage) {
    case KV_STORAGE_BF16: return back_dispatch<__nv_bfloat16, __nv_bfloat16>(plan, mode, a, z0, nzs);
    case KV_STORAGE_F16: return back_dispatch<__half, __half>(plan, mode, a, z0, nzs);
    default: return back_dispatch<float, float>(plan, mode, a, z0, nzs);
    }
}

kv_status exact_back_launch(kv_plan *plan, BackMode mode, const BackArgs &a) {
    return exact_back_slab_launch(plan, mode, a, 0, plan->g.nz);
}

kv_status exact_prescale_launch(kv_plan *plan, const float *y, void *yp) {
    ExGeom G = exgeom(plan, plan->g.n_views);
    dim3 block(32, 8), grid((G.nu + 31) / 32, (G.nv + 7) / 8, G.n_views);
    cudaStream_t st = plan->ctx->stream;
    LaunchTimer lt(plan->ctx, "prescale");
    switch (plan->storage) {
    case KV_STORAGE_BF16: prescale_kernel<__nv_bfloat16><<<grid, block, 0, st>>>(G, plan->ex, y, (__nv_bfloat16 *)yp); break;
    case KV_STORAGE_F16: prescale_kernel<__half><<<grid, block, 0, st>>>(G, plan->ex, y, (__half *)yp); break;
    default: prescale_kernel<float><<<grid, block, 0, st>>>(G, plan->ex, y, (float *)yp); break;
    }
    KV_CHECK_LAUNCH(plan->ctx, "prescale_kernel");
    return KV_OK;
}

// A^T 1 with FP64 accumulation.  Uses the plan's ratio workspace (float32
// view) for the ray factors.
kv_status exact_sensitivity_launch(kv_plan *plan, double *sens) {
    ExGeom G = exgeom(plan, plan->g.n_views);
    cudaStream_t st = plan->ctx->stream;
    float *ls = nullptr;
    KV_CHECK_CUDA(plan->ctx, cudaMallocAsync((void **)&ls, plan->nproj * sizeof(float), st));
    {
        dim3 block(32, 8), grid((G.nu + 31) / 32, (G.nv + 7) / 8, G.n_views);
        LaunchTimer lt(plan->ctx, "prescale");
        prescale_kernel<float><<<grid, block, 0, st>>>(G, plan->ex, nullptr, ls);
    }
    BackArgs a{ls, nullptr, nullptr, 1.f};
    dim3 block(32, plan->back_by);
    dim3 grid((G.nx + 31) / 32, (G.ny + plan->back_by - 1) / plan->back_by, G.nz);
    {
        LaunchTimer lt(plan->ctx, "exact_back_sens_f64");
        if (plan->back_rows > 0)
            back_r_dispatch<float, float, ACC_DF>(plan->back_rows, plan->back_slices, G, plan->ex, BACK_PLAIN, a, sens, 0, G.nz, st);
        else
            exact_back_kernel<float, float, ACC_DF, BACK_PLAIN><<<grid, block, 0, st>>>(G, plan->ex, a, sens, 0);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(ls, st);
    if (e != cudaSuccess) return kv_fail(plan->ctx, KV_ERR_CUDA, "sensitivity launch: %s", cudaGetErrorString(e));
    return KV_OK;
}

// ---------------------------------------------------------------------------
// Residual without device allocation
// ---------------------------------------------------------------------------
// kv_residual allocates its per-block partial sums for every call.  Callers
// that may not allocate device memory when they need a residual -- real-time
// loops that must not touch the allocator, or hosts whose device memory is
// owned by another framework's allocator or a fixed budget -- use
// kv_residual_noalloc instead.  Its scratch is this file-scope array: one FP64
// triple per forward block (at most KV_NOALLOC_MAX_BLOCKS blocks) and the
// final three sums, 1.5 MiB that every GPU loading the library holds until
// the process exits.  Every call overwrites the partials it reads, so nothing
// has to be cleared between calls; calls that overlap on one GPU share the
// array and race.
static __device__ __align__(256) double g_noalloc_scratch[3 * KV_NOALLOC_MAX_BLOCKS + 4];

namespace {
std::mutex g_noalloc_mutex;
// Device address of g_noalloc_scratch, per device ordinal: valid for the life
// of that device's primary context (the library never resets a device).
double *g_noalloc_ptr[64] = {};

// Set-up, once per device, with that device current: the host-side name of a
// __device__ array is not a device address; ask the runtime for it.
kv_status noalloc_scratch(kv_ctx *ctx, double **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    const int dev = ctx->device;
    if (dev < 0 || dev >= 64) return kv_fail(ctx, KV_ERR_INVALID_ARG, "device ordinal %d out of range", dev);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return kv_fail(ctx, KV_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return KV_OK;
}
}  // namespace

extern "C" kv_status kv_residual_noalloc(kv_plan *plan, const float *projections, const float *volume,
                                         double *rel_residual, double *loglik) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    kv_ctx *ctx = plan->ctx;
    if (projections == nullptr || volume == nullptr)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_residual_noalloc: null device buffer");
    if (plan->family != KV_FAMILY_EXACT || plan->storage != KV_STORAGE_F32)
        return kv_fail(ctx, KV_ERR_UNSUPPORTED, "kv_residual_noalloc: EXACT family with FP32 storage only");
    const int by = plan->fwd_by;
    if (by < 1 || by > 8) return kv_fail(ctx, KV_ERR_INVALID_ARG, "bad forward block");
    const size_t nblocks = (size_t)((plan->g.nu + 31) / 32) * ((plan->g.nv + by - 1) / by) * plan->g.n_views;
    if (nblocks > KV_NOALLOC_MAX_BLOCKS)
        return kv_fail(ctx, KV_ERR_INVALID_ARG,
                       "kv_residual_noalloc: this geometry needs %zu partial sums but the static scratch holds "
                       "%d (at most %d forward blocks of 32 x %d rays); use kv_residual",
                       nblocks, KV_NOALLOC_MAX_BLOCKS, KV_NOALLOC_MAX_BLOCKS, by);
    int caller_device = 0;
    KV_CHECK_CUDA(ctx, cudaGetDevice(&caller_device));
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    // the caller's current device is put back on every path out
    struct RestoreDevice {
        int dev;
        ~RestoreDevice() { cudaSetDevice(dev); }
    } restore{caller_device};
    double *scratch = nullptr;
    KV_TRY(noalloc_scratch(ctx, &scratch));
    double *partials = scratch, *sums = scratch + 3 * (size_t)KV_NOALLOC_MAX_BLOCKS;
    ExGeom G = exgeom(plan, plan->g.n_views);
    dim3 block(32, by), grid((G.nu + 31) / 32, (G.nv + by - 1) / by, G.n_views);
    FwdArgs a{volume, projections, nullptr, nullptr, 1.f};
    exact_fwd_kernel<float, float, FWD_RESID><<<grid, block, 0, ctx->stream>>>(G, plan->ex, a, partials);
    KV_CHECK_LAUNCH(ctx, "exact_fwd_kernel (no-alloc residual)");
    reduce_partials_kernel<<<1, 1024, 0, ctx->stream>>>(partials, nblocks, sums);
    KV_CHECK_LAUNCH(ctx, "reduce_partials_kernel (no-alloc residual)");
    double h[3];
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(h, sums, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (rel_residual) *rel_residual = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    if (loglik) *loglik = h[2];
    return KV_OK;
}

// ---------------------------------------------------------------------------
// Batched solves: many EXACT reconstructions of uneven size in one launch
// ---------------------------------------------------------------------------
// The forward and the backprojection of every problem are cut into the same
// tiles the per-plan kernels use.  A persistent kernel (a few CTAs per SM)
// pulls tile indices from a device counter and finds the problem of each tile
// by binary search over the problems' first tile indices, then runs the very
// same tile function: results are bit-identical to solving one by one.
namespace {

struct BatchItem {
    ExGeom G;
    ExactTables T;
    const float *p;        // measured projections
    float *x;              // iterate (updated in place)
    float *ratio;          // forward output: Ls * relax * p / Ax
    const double *sens;    // A^T 1
    int ftx, fty;          // forward tiles per view (u, v)
    int btx, bty;          // backprojection tiles per slice (i, j)
    long long f0, b0;      // first forward / backprojection tile of this problem
};

__device__ __forceinline__ int batch_find(const BatchItem *items, int n, long long tile, bool fwd) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const long long start = fwd ? items[mid].f0 : items[mid].b0;
        if (start <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256) batch_fwd_kernel(const BatchItem *__restrict__ items, int n,
                                                        long long total, unsigned long long *counter,
                                                        float relax) {
    __shared__ long long s_tile;
    while (true) {
        if (threadIdx.x == 0 && threadIdx.y == 0) s_tile = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long tile = s_tile;
        __syncthreads();
        if (tile >= total) return;
        const BatchItem &B = items[batch_find(items, n, tile, true)];
        const long long local = tile - B.f0;
        const long long per_view = (long long)B.ftx * B.fty;
        const int p = (int)(local / per_view);
        const int rem = (int)(local % per_view);
        FwdArgs a{B.x, B.p, B.ratio, nullptr, relax};
        fwd_tile<float, float, FWD_MLEM>(B.G, B.T, a, nullptr, rem % B.ftx, rem / B.ftx, p, 0);
    }
}

__global__ void __launch_bounds__(256) batch_back_kernel(const BatchItem *__restrict__ items, int n,
                                                         long long total, unsigned long long *counter,
                                                         float relax) {
    __shared__ long long s_tile;
    while (true) {
        if (threadIdx.x == 0 && threadIdx.y == 0) s_tile = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long tile = s_tile;
        __syncthreads();
        if (tile >= total) return;
        const BatchItem &B = items[batch_find(items, n, tile, false)];
        const long long local = tile - B.b0;
        const long long per_slice = (long long)B.btx * B.bty;
        const int k = (int)(local / per_slice);
        const int rem = (int)(local % per_slice);
        BackArgs a{B.ratio, B.x, B.sens, relax};
        back_tile<float, float, ACC_F32, BACK_MLEM>(B.G, B.T, a, nullptr, rem % B.btx, rem / B.btx, k);
        __syncwarp();
    }
}

}  // namespace

// Captures `iters` MLEM iterations over all problems as one CUDA graph and
// launches it on the context stream.  Plans must be EXACT / FP32 with their
// sensitivity images computed and ratio workspaces allocated; p[i] / x[i] are
// device buffers.  Block shape: 32 x by (forward) and 32 x bb (backprojection).
kv_status exact_batch_mlem_launch(kv_ctx *ctx, int n, kv_plan *const *plans, const float *const *p,
                                  float *const *x, int iters, float relax, int by, int bb) {
    std::vector<BatchItem> items(n);
    long long f = 0, b = 0;
    for (int i = 0; i < n; ++i) {
        const kv_plan *pl = plans[i];
        BatchItem &it = items[i];
        it.G = exgeom(pl, pl->g.n_views);
        it.T = pl->ex;
        it.p = p[i];
        it.x = x[i];
        it.ratio = static_cast<float *>(pl->d_ratio);
        it.sens = pl->d_sens;
        it.ftx = (pl->g.nu + 31) / 32;
        it.fty = (pl->g.nv + by - 1) / by;
        it.btx = (pl->g.nx + 31) / 32;
        it.bty = (pl->g.ny + bb - 1) / bb;
        it.f0 = f;
        it.b0 = b;
        f += (long long)it.ftx * it.fty * pl->g.n_views;
        b += (long long)it.btx * it.bty * pl->g.nz;
    }
    cudaStream_t cap = ctx->own_stream;
    BatchItem *d_items = nullptr;
    unsigned long long *d_counter = nullptr;
    KV_CHECK_CUDA(ctx, cudaMalloc((void **)&d_items, n * sizeof(BatchItem)));
    kv_status s = KV_OK;
    if (cudaMalloc((void **)&d_counter, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(d_items);
        return kv_fail(ctx, KV_ERR_OOM, "batch counters");
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int occ_f = 0, occ_b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, batch_fwd_kernel, 32 * by, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, batch_back_kernel, 32 * bb, 0);
    const int grid_f = ctx->sm_count * (occ_f > 0 ? occ_f : 1);
    const int grid_b = ctx->sm_count * (occ_b > 0 ? occ_b : 1);
    do {
        if (cudaMemcpyAsync(d_items, items.data(), n * sizeof(BatchItem), cudaMemcpyHostToDevice, ctx->stream) !=
            cudaSuccess) { s = kv_fail(ctx, KV_ERR_CUDA, "batch descriptor upload"); break; }
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) { s = kv_fail(ctx, KV_ERR_CUDA, "batch sync"); break; }
        if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            s = kv_fail(ctx, KV_ERR_CUDA, "batch graph capture");
            break;
        }
        for (int it = 0; it < iters; ++it) {
            cudaMemsetAsync(d_counter, 0, 2 * sizeof(unsigned long long), cap);
            batch_fwd_kernel<<<grid_f, dim3(32, by), 0, cap>>>(d_items, n, f, d_counter, relax);
            batch_back_kernel<<<grid_b, dim3(32, bb), 0, cap>>>(d_items, n, b, d_counter + 1, relax);
        }
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        if (e != cudaSuccess) { s = kv_fail(ctx, KV_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e)); break; }
        e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) { s = kv_fail(ctx, KV_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); break; }
        LaunchTimer lt(ctx, "batch_mlem_graph");
        e = cudaGraphLaunch(exec, ctx->stream);
        if (e != cudaSuccess) { s = kv_fail(ctx, KV_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e)); break; }
    } while (0);
    cudaStreamSynchronize(ctx->stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaFree(d_items);
    cudaFree(d_counter);
    return s;
}

// ---------------------------------------------------------------------------
// Autotuner: ray-bundle and voxel-tile shapes
// ---------------------------------------------------------------------------
namespace {

template <typename VolT, typename ProjT>
float time_fwd(kv_ctx *ctx, const ExGeom &G, const ExactTables &T, const void *vol, void *out, int by,
               cudaEvent_t e0, cudaEvent_t e1) {
    dim3 block(32, by), grid((G.nu + 31) / 32, (G.nv + by - 1) / by, G.n_views);
    FwdArgs a{vol, nullptr, out, nullptr, 1.f};
    float best = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(e0, ctx->stream);
        exact_fwd_kernel<VolT, ProjT, FWD_PLAIN><<<grid, block, 0, ctx->stream>>>(G, T, a, nullptr);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    return best;
}

template <typename VolT, typename ProjT, int ACC>
float time_back(kv_ctx *ctx, const ExGeom &G, const ExactTables &T, const void *yp, void *vol, int bb,
                cudaEvent_t e0, cudaEvent_t e1) {
    dim3 block(32, bb), grid((G.nx + 31) / 32, (G.ny + bb - 1) / bb, G.nz);
    BackArgs a{yp, vol, nullptr, 1.f};
    float best = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(e0, ctx->stream);
        exact_back_kernel<VolT, ProjT, ACC, BACK_PLAIN><<<grid, block, 0, ctx->stream>>>(G, T, a, nullptr, 0);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    return best;
}

template <typename VolT, typename ProjT, int ACC>
void tune(kv_ctx *ctx, const ExGeom &G, const ExactTables &T, void *vol, void *proj, int &fwd_by, int &back_by) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int by : {1, 2, 4, 8}) {
        const float ms = time_fwd<VolT, ProjT>(ctx, G, T, vol, proj, by, e0, e1);
        if (ms < best) { best = ms; fwd_by = by; }
    }
    best = 1e30f;
    for (int bb : {2, 4, 8}) {   // 256 threads per block at most
        const float ms = time_back<VolT, ProjT, ACC>(ctx, G, T, proj, vol, bb, e0, e1);
        if (ms < best) { best = ms; back_by = bb; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

// Median of three timed calls of fn after one untimed call, in ms.
template <typename F>
float median3(kv_ctx *ctx, cudaEvent_t e0, cudaEvent_t e1, F fn) {
    fn();
    float t[3];
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0, ctx->stream);
        fn();
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&t[r], e0, e1);
    }
    std::sort(t, t + 3);
    return t[1];
}

// The shapes the tuner picked for one geometry shape and storage.
struct TuneResult {
    int fwd_by, back_by;
    FwdSlabCfg fslab;
    int back_rows, back_slices;
    BackStageCfg bstage;
};

std::mutex g_tune_mutex;
std::vector<std::pair<std::vector<long long>, TuneResult>> g_tune_cache;

// The slab forward shapes and gather backprojector shapes, timed through the
// plan's own launchers on its first (at most) 12 views.
template <typename VolT, typename ProjT, int ACC>
kv_status tune_shapes(kv_plan *plan, int P, TuneResult &best) {
    kv_ctx *ctx = plan->ctx;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const kv_geometry &g = plan->g;
    float bt = 1e30f;
    static const int shapes[][3] = {{8, 4, 2}, {4, 4, 3}, {8, 2, 2}, {4, 2, 3}, {2, 4, 3}};
    const int group = fwd_slab_default_group(g.n_views);
    const FwdSlabCfg keep = plan->fslab;
    const FwdArgs fa{plan->d_vol, nullptr, plan->d_ratio, nullptr, 1.f};
    for (const auto &sh : shapes) {
        FwdSlabCfg c;
        if (!fwd_slab_fit(plan, sh[0], sh[1], sh[2], group, &c, nullptr)) continue;
        plan->fslab = c;
        const float ms = median3(ctx, e0, e1, [&] { exact_forward_launch(plan, plan->ex, P, FWD_PLAIN, fa); });
        if (ms < bt) {
            bt = ms;
            best.fslab = c;
        }
    }
    plan->fslab = keep;
    // gather backprojector: (rows, slices) per thread, or one voxel per thread
    const ExGeom G = exgeom(plan, P);
    const BackArgs ba{plan->d_ratio, plan->d_vol, nullptr, 1.f};
    static const int bshapes[][2] = {{8, 1}, {4, 1}, {4, 2}, {2, 1}, {2, 2}, {1, 1}};
    bt = 1e30f;
    for (const auto &sh : bshapes) {
        const float ms = median3(ctx, e0, e1, [&] {
            back_r_dispatch<VolT, ProjT, ACC>(sh[0], sh[1], G, plan->ex, BACK_PLAIN, ba, nullptr, 0, g.nz, ctx->stream);
        });
        if (ms < bt) {
            bt = ms;
            best.back_rows = sh[0];
            best.back_slices = sh[1];
        }
    }
    {
        dim3 block(32, best.back_by), grid((G.nx + 31) / 32, (G.ny + best.back_by - 1) / best.back_by, g.nz);
        const float ms = median3(ctx, e0, e1, [&] {
            exact_back_kernel<VolT, ProjT, ACC, BACK_PLAIN><<<grid, block, 0, ctx->stream>>>(G, plan->ex, ba, nullptr, 0);
        });
        if (ms < bt) {
            bt = ms;
            best.back_rows = 0;
            best.back_slices = 1;
        }
    }
    // the staged backprojector (FP32 storage), used instead when it is faster
    best.bstage = BackStageCfg{};
    if constexpr (std::is_same<VolT, float>::value && ACC == ACC_F32) {
        static const int sshapes[][2] = {{8, 2}, {4, 2}, {4, 3}};
        const BackStageCfg keep_stage = plan->bstage;
        for (const auto &sh : sshapes) {
            BackStageCfg c;
            if (!back_stage_fit(plan, sh[0], sh[1], &c, nullptr)) continue;
            plan->bstage = c;
            const float ms = median3(ctx, e0, e1, [&] { back_stage_launch(plan, BACK_PLAIN, ba, 0, g.nz, P); });
            if (ms < bt) {
                bt = ms;
                best.bstage = c;
            }
        }
        plan->bstage = keep_stage;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    return KV_OK;
}

}  // namespace

// Times the candidate shapes on the plan's own tables with a subset of its
// views (at most 6: the cost per view is nearly uniform), on zero-filled
// buffers (the Siddon walk does not depend on the values).
kv_status exact_autotune(kv_plan *plan) {
    kv_ctx *ctx = plan->ctx;
    const kv_geometry &g = plan->g;
    const std::vector<long long> key = {g.nx, g.ny, g.nz, g.nu, g.nv, g.n_views, (long long)plan->storage};
    auto apply = [plan](const TuneResult &r) {
        plan->fwd_by = r.fwd_by;
        plan->back_by = r.back_by;
        plan->fslab = r.fslab;
        plan->back_rows = r.back_rows;
        plan->back_slices = r.back_slices;
        plan->bstage = r.bstage;
    };
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        for (const auto &e : g_tune_cache)
            if (e.first == key) {
                apply(e.second);
                return KV_OK;
            }
    }
    const size_t es = kv_storage_bytes(plan->storage);
    if (plan->d_vol == nullptr) KV_CHECK_CUDA(ctx, cudaMalloc(&plan->d_vol, plan->nvox * es));
    if (plan->d_ratio == nullptr) KV_CHECK_CUDA(ctx, cudaMalloc(&plan->d_ratio, plan->nproj * es));
    KV_CHECK_CUDA(ctx, cudaMemsetAsync(plan->d_vol, 0, plan->nvox * es, ctx->stream));
    KV_CHECK_CUDA(ctx, cudaMemsetAsync(plan->d_ratio, 0, plan->nproj * es, ctx->stream));
    const ExGeom G = exgeom(plan, g.n_views < 6 ? g.n_views : 6);
    TuneResult r{plan->fwd_by, plan->back_by, plan->fslab, plan->back_rows, plan->back_slices, plan->bstage};
    // one-thread-per-ray / per-voxel block heights (the fallback kernels)
    switch (plan->storage) {
    case KV_STORAGE_BF16: tune<__nv_bfloat16, __nv_bfloat16, ACC_F32>(ctx, G, plan->ex, plan->d_vol, plan->d_ratio, r.fwd_by, r.back_by); break;
    case KV_STORAGE_F16: tune<__half, __half, ACC_F32>(ctx, G, plan->ex, plan->d_vol, plan->d_ratio, r.fwd_by, r.back_by); break;
    default: tune<float, float, ACC_F32>(ctx, G, plan->ex, plan->d_vol, plan->d_ratio, r.fwd_by, r.back_by); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    // slab forward and gather backprojector shapes
    const int P = g.n_views < 12 ? g.n_views : 12;
    switch (plan->storage) {
    case KV_STORAGE_BF16: KV_TRY((tune_shapes<__nv_bfloat16, __nv_bfloat16, ACC_F32>(plan, P, r))); break;
    case KV_STORAGE_F16: KV_TRY((tune_shapes<__half, __half, ACC_F32>(plan, P, r))); break;
    default: KV_TRY((tune_shapes<float, float, ACC_F32>(plan, P, r))); break;
    }
    apply(r);
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache.emplace_back(key, r);
    return KV_OK;
}
