// kv_rc.cu -- RC family: the reference projector pair reproduced on sm_103a.
//
// Forward: source/modules/reconstruction/Projector.cu:227-372 (kernel) with
// FindProjectionAlphas_d Projector.cu:45-223.  Each ray's plane-crossing
// parameters form three ascending arithmetic sequences (x, y and z planes,
// each generated by repeated addition exactly as the reference fills its
// list) plus the entries the reference leaves at 1.0.  The reference sorts
// that list with an O(n^2) selection sort in 8 KB of thread-local memory;
// here the sorted order is produced by a four-way merge of the sequences in
// registers, which yields the same sorted values.  The segment midpoint is
// computed in double by the reference (Projector.cu:350-354); here it is
// evaluated in float and redone in double only when the float result lies
// within 1e-3 voxel of an integer, so the truncated index is the same.
//
// Backprojector: Projector.cu:376-785, one thread per voxel, an 11x11 window
// of pixel rays per view, weights normalised by their sum.  The x-plane
// parameters of the window's 11 columns are computed once per view instead of
// once per pixel (same values, same operations).
//
// This translation unit is compiled with -fmad=false: no multiply-add is
// fused, matching the reference kernel source compiled for the host, against
// which the results are bit-identical.
#include "kv_internal.h"

namespace {

struct RcGeom {
    int nx, ny, nz, nu, nv, n_views;
    float dx, dy, dz, du, dv;
};

__device__ __forceinline__ bool rc_sup_eq(float a, float b) {
    const float d = a - b;
    return a > b || (d < 0.0000001F && d > -0.0000001F);
}

// (int)((double)base + (double)c * (double)d), Projector.cu:352-354
__device__ __forceinline__ int rc_index(float base, float c, float d) {
    const float v = fmaf(c, d, base);
    const float r = rintf(v);
    if (fabsf(v - r) > fmaxf(1e-3f, fabsf(v) * 1e-6f)) return (int)v;
    const double dv = (double)base + (double)c * (double)d;
    return (int)dv;
}

struct Seq {
    float val, step;
    int left;
};

template <int MODE>
__global__ void __launch_bounds__(128) rc_forward_kernel(RcGeom G, const float *__restrict__ src,
                                                         const float *__restrict__ org,
                                                         const float *__restrict__ vol,
                                                         const float *__restrict__ meas,
                                                         float *__restrict__ out, float relax) {
    const int u = blockIdx.x * 32 + threadIdx.x;
    const int v = blockIdx.y * blockDim.y + threadIdx.y;
    const int p = blockIdx.z;
    if (u >= G.nu || v >= G.nv) return;
    const size_t ray = ((size_t)p * G.nv + v) * G.nu + u;
    const float tol = 0.000001F;
    const int n[3] = {G.nx, G.ny, G.nz};
    float s[3], d[3], half[3];
    s[0] = src[3 * p] / G.dx;
    s[1] = src[3 * p + 1] / G.dy;
    s[2] = src[3 * p + 2] / G.dz;
    const float px = (org[3 * p] + ((float)u + 0.5F) * G.du) / G.dx;
    const float py = (org[3 * p + 1] + ((float)v + 0.5F) * G.dv) / G.dy;
    const float pz = org[3 * p + 2] / G.dz;
    d[0] = px - s[0];
    d[1] = py - s[1];
    d[2] = pz - s[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) half[a] = (float)n[a] / 2.F;

    float mins[3], maxs[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float a1 = fabsf(d[a]) > tol ? (-half[a] - s[a]) / d[a] : 0.F;
        const float aN = fabsf(d[a]) > tol ? (half[a] - s[a]) / d[a] : 0.F;
        mins[a] = fminf(a1, aN);
        maxs[a] = fmaxf(a1, aN);
    }
    const float amin = fmaxf(fmaxf(0.F, mins[0]), fmaxf(mins[1], mins[2]));
    const float amax = fminf(fminf(1.F, maxs[0]), fminf(maxs[1], maxs[2]));
    float q = 0.F;
    if (!rc_sup_eq(amin, amax)) {
        Seq sq[3];
        int total = 3, filled = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float at_hi = d[a] > 0 ? amax : amin;
            const float at_lo = d[a] > 0 ? amin : amax;
            const float up = (half[a] + s[a]) + at_hi * d[a];
            const int mx = max(0, min(n[a] - 1, (int)up));
            const float dn = (half[a] - s[a]) - at_lo * d[a];
            const int mn = max(0, min(mx, n[a] - (int)dn));
            const int span = mx - mn;
            total += span;
            const int count = a < 2 ? span + 1 : (span >= 2 ? span - 1 : 1);
            if (fabsf(d[a]) > tol) {
                const float step = 1.F / d[a];
                const float plane = (float)(d[a] > 0 ? mn : mx);
                sq[a].val = step * ((-half[a] - s[a]) + plane);
                sq[a].step = fabsf(step);
                sq[a].left = count;
                filled += count;
            } else {
                sq[a].val = 0.F;
                sq[a].step = 0.F;
                sq[a].left = 0;
            }
        }
        int ones = total - filled;   // entries left at the fill value 1.0
        const float b0 = half[0] + s[0], b1 = half[1] + s[1], b2 = half[2] + s[2];
        const float d0 = d[0], d1 = d[1], d2 = d[2];
        // the three sequences as scalars (a dynamically indexed array would
        // live in local memory and every merge step would go through L1)
        float v0 = sq[0].val, v1 = sq[1].val, v2 = sq[2].val;
        const float st0 = sq[0].step, st1 = sq[1].step, st2 = sq[2].step;
        int l0 = sq[0].left, l1 = sq[1].left, l2 = sq[2].left;
        float acc = 0.F, wsum = 0.F;
        float prev = 0.F;
        for (int e = 0; e < total; ++e) {
            // pop the smallest head among x, y, z and the 1.0 entries
            float best = 3.402823466e38F;
            int which = 3;
            if (l0 > 0) { best = v0; which = 0; }
            if (l1 > 0 && v1 < best) { best = v1; which = 1; }
            if (l2 > 0 && v2 < best) { best = v2; which = 2; }
            if (ones > 0 && 1.0F < best) { best = 1.0F; which = 3; }
            if (which == 0) {
                v0 = v0 + st0;
                --l0;
            } else if (which == 1) {
                v1 = v1 + st1;
                --l1;
            } else if (which == 2) {
                v2 = v2 + st2;
                --l2;
            } else if (ones > 0) {
                --ones;
            }
            if (e > 0) {
                const float c = (best + prev) * 0.5F;
                const int ix = rc_index(b0, c, d0);
                const int iy = rc_index(b1, c, d1);
                const int iz = rc_index(b2, c, d2);
                const float w = best - prev;
                if (ix >= 0 && ix < G.nx && iy >= 0 && iy < G.ny && iz >= 0 && iz < G.nz && w > tol) {
                    const size_t idx = ((size_t)iz * G.ny + iy) * G.nx + ix;
                    wsum += w;
                    acc += w * __ldg(vol + idx);
                }
            }
            prev = best;
        }
        q = wsum > tol ? acc / wsum : 0.F;
    }
    if (MODE == RC_PLAIN) {
        out[ray] = q;
    } else if (MODE == RC_MLEM) {
        // Reconstructors.h:207-213: ratio where q != 0 (AlmostEqualRelative)
        out[ray] = q != 0.F ? relax * (meas[ray] / q) : q;
    } else {
        // Reconstructors.h:90-93
        out[ray] = relax * (meas[ray] - q);
    }
}

template <int MODE>
__global__ void __launch_bounds__(128) rc_back_kernel(RcGeom G, const float *__restrict__ src,
                                                      const float *__restrict__ org,
                                                      const float *__restrict__ proj,
                                                      float *__restrict__ vol, int z0) {
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = z0 + (int)blockIdx.z;   // slices z0 .. z0 + gridDim.z - 1
    if (x >= G.nx || y >= G.ny) return;
    const float tol = 0.000000000000000000000001F;
    const int semi = 5;
    const float vfx = (float)x - (float)G.nx / 2.F;
    const float vfy = (float)y - (float)G.ny / 2.F;
    const float vfz = (float)z - (float)G.nz / 2.F;
    float acc = 0.F, wsum = 0.F;
    for (int p = 0; p < G.n_views; ++p) {
        const float ox = org[3 * p], oy = org[3 * p + 1], oz = org[3 * p + 2];
        const float sx = src[3 * p] / G.dx, sy = src[3 * p + 1] / G.dy, sz = src[3 * p + 2] / G.dz;
        const float ofx = ox / G.dx, ofy = oy / G.dy, ofz = oz / G.dz;
        const float ex = (ox + (float)G.nu * G.du) / G.dx;
        const float ey = (oy + (float)G.nv * G.dv) / G.dy;
        const float rx = (vfx + 0.5F) - sx, ry = (vfy + 0.5F) - sy, rz = (vfz + 0.5F) - sz;
        const float az = fabsf(rz) > tol ? (ofz - sz) / rz : 0.F;
        const float hx = sx + rx * az, hy = sy + ry * az;
        const float mx = (float)semi * G.du / G.dx, my = (float)semi * G.dv / G.dy;
        if (!(hx > ofx - mx && hx < ex + mx && hy > ofy - my && hy < ey + my)) continue;
        const int pxl = (int)((hx - ofx) * G.dx / G.du);
        const int pyl = (int)((hy - ofy) * G.dy / G.dv);
        int x0 = pxl - semi, x1 = pxl + semi, y0 = pyl - semi, y1 = pyl + semi;
        x0 = x0 < 0 ? 0 : (x0 >= G.nu ? G.nu - 1 : x0);
        x1 = x1 < 0 ? 0 : (x1 >= G.nu ? G.nu - 1 : x1);
        y0 = y0 < 0 ? 0 : (y0 >= G.nv ? G.nv - 1 : y0);
        y1 = y1 < 0 ? 0 : (y1 >= G.nv ? G.nv - 1 : y1);
        const float dzr = oz / G.dz - sz;
        const float a1z = fabsf(dzr) > tol ? (vfz - sz) / dzr : 0.F;
        const float a2z = fabsf(dzr) > tol ? (vfz + 1.F - sz) / dzr : 0.F;
        const float mnz = fminf(a1z, a2z), mxz = fmaxf(a1z, a2z);
        // x parameters of the window columns (at most 11)
        float cmn[11], cmx[11];
#pragma unroll
        for (int c = 0; c < 11; ++c) {
            const int qx = x0 + c;
            const float dxr = (ox + ((float)qx + 0.5F) * G.du) / G.dx - sx;
            const float a1x = fabsf(dxr) > tol ? (vfx - sx) / dxr : 0.F;
            const float a2x = fabsf(dxr) > tol ? (vfx + 1.F - sx) / dxr : 0.F;
            cmn[c] = fmaxf(0.F, fminf(a1x, a2x));
            cmx[c] = fminf(1.F, fmaxf(a1x, a2x));
        }
        const float *pv = proj + (size_t)p * G.nu * G.nv;
        const int ncol = x1 - x0 + 1;
        for (int qy = y0; qy <= y1; ++qy) {
            const float dyr = (oy + ((float)qy + 0.5F) * G.dv) / G.dy - sy;
            const float a1y = fabsf(dyr) > tol ? (vfy - sy) / dyr : 0.F;
            const float a2y = fabsf(dyr) > tol ? (vfy + 1.F - sy) / dyr : 0.F;
            const float lo_r = fmaxf(fminf(a1y, a2y), mnz);
            const float hi_r = fminf(fmaxf(a1y, a2y), mxz);
            const float *row = pv + (size_t)qy * G.nu + x0;
#pragma unroll
            for (int c = 0; c < 11; ++c) {
                if (c < ncol) {
                    const float lo = fmaxf(cmn[c], lo_r);
                    const float hi = fminf(cmx[c], hi_r);
                    if (rc_sup_eq(hi, lo)) {
                        const float w = hi - lo;
                        if (w > tol) {
                            wsum += w;
                            acc += w * __ldg(row + c);
                        }
                    }
                }
            }
        }
    }
    const float b = wsum > tol ? acc / wsum : 0.F;
    const size_t idx = ((size_t)z * G.ny + y) * G.nx + x;
    if (MODE == RC_PLAIN) vol[idx] = b;
    else if (MODE == RC_MLEM) vol[idx] = vol[idx] * b;     // Reconstructors.h:238-241
    else vol[idx] = vol[idx] + b;                          // Reconstructors.h:118-121
}

// Elementwise ratio step of recons::MLEM / recons::ART on a forward result q,
// the same float operations as the fused epilogue of rc_forward_kernel.
__global__ void rc_ratio_kernel(int mode, const float *__restrict__ p, float *__restrict__ q, size_t n,
                                float relax) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float qi = q[i];
        q[i] = mode == RC_MLEM ? (qi != 0.F ? relax * (p[i] / qi) : qi) : relax * (p[i] - qi);
    }
}

RcGeom rcgeom(const kv_plan *plan, int n_views) {
    const kv_geometry &g = plan->g;
    return RcGeom{g.nx, g.ny, g.nz, g.nu, g.nv, n_views, g.dx, g.dy, g.dz, g.du, g.dv};
}

}  // namespace

kv_status rc_forward_launch(kv_plan *plan, const float *d_src, const float *d_org, int n_views,
                            int mode, const float *vol, const float *meas, float *out, float relax) {
    RcGeom G = rcgeom(plan, n_views);
    dim3 block(32, 4), grid((G.nu + 31) / 32, (G.nv + 3) / 4, n_views);
    cudaStream_t st = plan->ctx->stream;
    LaunchTimer lt(plan->ctx, "rc_fwd");
    switch (mode) {
    case RC_PLAIN: rc_forward_kernel<RC_PLAIN><<<grid, block, 0, st>>>(G, d_src, d_org, vol, meas, out, relax); break;
    case RC_MLEM: rc_forward_kernel<RC_MLEM><<<grid, block, 0, st>>>(G, d_src, d_org, vol, meas, out, relax); break;
    default: rc_forward_kernel<RC_ART><<<grid, block, 0, st>>>(G, d_src, d_org, vol, meas, out, relax); break;
    }
    KV_CHECK_LAUNCH(plan->ctx, "rc_forward_kernel");
    return KV_OK;
}

kv_status rc_back_slab_launch(kv_plan *plan, int mode, const float *proj, float *vol, int z0, int nzs) {
    if (z0 < 0 || nzs < 1 || z0 + nzs > plan->g.nz)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "bad slice range for the backprojection");
    RcGeom G = rcgeom(plan, plan->g.n_views);
    dim3 block(32, 4), grid((G.nx + 31) / 32, (G.ny + 3) / 4, nzs);
    cudaStream_t st = plan->ctx->stream;
    LaunchTimer lt(plan->ctx, "rc_back");
    switch (mode) {
    case RC_PLAIN: rc_back_kernel<RC_PLAIN><<<grid, block, 0, st>>>(G, plan->d_src, plan->d_org, proj, vol, z0); break;
    case RC_MLEM: rc_back_kernel<RC_MLEM><<<grid, block, 0, st>>>(G, plan->d_src, plan->d_org, proj, vol, z0); break;
    default: rc_back_kernel<RC_ART><<<grid, block, 0, st>>>(G, plan->d_src, plan->d_org, proj, vol, z0); break;
    }
    KV_CHECK_LAUNCH(plan->ctx, "rc_back_kernel");
    return KV_OK;
}

kv_status rc_back_launch(kv_plan *plan, int mode, const float *proj, float *vol) {
    return rc_back_slab_launch(plan, mode, proj, vol, 0, plan->g.nz);
}

kv_status residual_reduce_launch(kv_ctx *ctx, const float *q, const float *p, size_t n, double *red);

kv_status rc_residual_launch(kv_plan *plan, const float *q, const float *p, double *red) {
    return residual_reduce_launch(plan->ctx, q, p, plan->nproj, red);
}

kv_status rc_ratio_launch(kv_plan *plan, int mode, const float *p, float *q, float relax) {
    const int grid = plan->ctx->sm_count > 0 ? plan->ctx->sm_count * 8 : 1024;
    LaunchTimer lt(plan->ctx, "rc_ratio");
    rc_ratio_kernel<<<grid, 256, 0, plan->ctx->stream>>>(mode, p, q, plan->nproj, relax);
    KV_CHECK_LAUNCH(plan->ctx, "rc_ratio_kernel");
    return KV_OK;
}
