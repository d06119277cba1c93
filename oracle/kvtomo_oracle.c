/*
 * kvtomo_oracle.c -- CPU ORACLE for the kvtomo engine.  TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
 * legs may load this library; the engine itself never calls it.  It restates,
 * on the host, every operator the CUDA path computes:
 *
 *   RC family (reference compatible, FP32).  Restatement of the Kevernals
 *   kernels source/modules/reconstruction/Projector.cu:
 *     kvo_rc_forward  <- CudaPerformProjection  Projector.cu:227-372 with
 *                        FindProjectionAlphas_d Projector.cu:45-223
 *     kvo_rc_back     <- CudaPerformBackProjection Projector.cu:376-785
 *   and of the host drivers source/modules/reconstruction/Reconstructors.h:
 *     kvo_rc_mlem     <- recons::MLEM Reconstructors.h:136-253
 *     kvo_rc_art      <- recons::ART  Reconstructors.h:19-134
 *     kvo_saa_shifts  <- recons::ShiftAndAdd shift rule Reconstructors.h:287-331
 *     kvo_saa         <- the zero-pad / extract / weighted-sum pipeline
 *                        Reconstructors.h:336-378 (VTK filters, restated)
 *   Float operations follow the reference's expression order; the library is
 *   built with -ffp-contract=off so no multiply-add is fused, which makes it
 *   bit-identical to the reference kernel source compiled for the host.
 *
 *   EXACT family (FP64).  Textbook Siddon ray tracing (R. L. Siddon, Med.
 *   Phys. 12(2), 1985; incremental form of F. Jacobs et al., 1998): the
 *   line integral of a voxelised volume and its transpose, computed from the
 *   merged list of plane crossings.  It shares no code or parametrisation with
 *   the GPU kernels, which use a per-slice local parametrisation.
 *
 *   Phantom: seeded ellipsoid rasteriser (float, fixed operation order).
 *
 * Parity of the RC restatement is pinned against the reference kernels
 * compiled from the reference tree (oracle/build_ref.sh); the EXACT oracle is
 * pinned by known-answer tests (chord lengths, impulse responses).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Same layout as kv_geometry in include/kvtomo.h. */
typedef struct kvo_geom {
    int32_t nx, ny, nz;
    float dx, dy, dz;
    int32_t n_views;
    int32_t nu, nv;
    float du, dv;
    const float *src;
    const float *det_origin;
    float fulcrum_z;
} kvo_geom;

int kvo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void kvo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ======================================================================
 * RC family
 * ====================================================================== */

/* floatEq / floatSupEq with the reference's default tolerance 1e-7
 * (Projector.cu:22-37). */
static int rc_float_eq(float a, float b, float tol) {
    if (tol < 0) return (a - b) < -tol && (a - b) > tol;
    return (a - b) < tol && (a - b) > -tol;
}
static int rc_float_sup_eq(float a, float b) { return a > b || rc_float_eq(a, b, 0.0000001F); }

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

static int cmp_float(const void *pa, const void *pb) {
    float a = *(const float *)pa, b = *(const float *)pb;
    return (a > b) - (a < b);
}

/* Ray set-up of Projector.cu:301-323, in floating-voxel units. */
static void rc_ray_setup(const kvo_geom *g, int view, int u, int v, float s[3], float d[3]) {
    const float *sp = g->src + 3 * view, *op = g->det_origin + 3 * view;
    const float spacing[3] = {g->dx, g->dy, g->dz};
    float pix[3];
    for (int a = 0; a < 3; ++a) s[a] = sp[a] / spacing[a];
    pix[0] = (op[0] + ((float)u + 0.5F) * g->du) / g->dx;
    pix[1] = (op[1] + ((float)v + 0.5F) * g->dv) / g->dy;
    pix[2] = op[2] / g->dz;
    for (int a = 0; a < 3; ++a) d[a] = pix[a] - s[a];
}

/* Returns 0 when the ray misses the volume box (the reference returns no
 * value there, Projector.cu:79-85; the ray is then written as 0, :273). */
int kvo_rc_ray_hits(const kvo_geom *g, int view, int u, int v) {
    const int n[3] = {g->nx, g->ny, g->nz};
    const float tol = 0.000001F;
    float s[3], d[3], lo = 0.F, hi = 1.F;
    rc_ray_setup(g, view, u, v, s, d);
    float mins[3], maxs[3];
    for (int a = 0; a < 3; ++a) {
        float half = (float)n[a] / 2.F;
        float a1 = fabsf(d[a]) > tol ? (-half - s[a]) / d[a] : 0.F;
        float aN = fabsf(d[a]) > tol ? (half - s[a]) / d[a] : 0.F;
        mins[a] = fminf(a1, aN);
        maxs[a] = fmaxf(a1, aN);
    }
    lo = fmaxf(fmaxf(0.F, mins[0]), fmaxf(mins[1], mins[2]));
    hi = fminf(fminf(1.F, maxs[0]), fminf(maxs[1], maxs[2]));
    return !rc_float_sup_eq(lo, hi);
}

/* Textbook selection sort, the ordering step the reference uses
 * (Projector.cu:204-220): O(n^2) compares.  Only used to time the reference's
 * CPU cost; qsort gives the same sorted values. */
static void selection_sort(float *a, unsigned n) {
    for (unsigned i = 0; i + 1 < n; ++i) {
        unsigned m = i;
        for (unsigned j = i + 1; j < n; ++j)
            if (a[j] < a[m]) m = j;
        float t = a[m];
        a[m] = a[i];
        a[i] = t;
    }
}

/* One ray of the RC forward operator.  `alphas` is scratch of >= 4096 floats.
 * ref_sort != 0 orders the list with the reference's selection sort. */
static float rc_forward_ray_sorted(const kvo_geom *g, const float *vol, int view, int u, int v,
                                   float *alphas, int ref_sort) {
    const int n[3] = {g->nx, g->ny, g->nz};
    const float tol = 0.000001F;
    float s[3], d[3], half[3];
    rc_ray_setup(g, view, u, v, s, d);
    for (int a = 0; a < 3; ++a) half[a] = (float)n[a] / 2.F;

    /* box clip, Projector.cu:53-85 */
    float mins[3], maxs[3];
    for (int a = 0; a < 3; ++a) {
        float a1 = fabsf(d[a]) > tol ? (-half[a] - s[a]) / d[a] : 0.F;
        float aN = fabsf(d[a]) > tol ? (half[a] - s[a]) / d[a] : 0.F;
        mins[a] = fminf(a1, aN);
        maxs[a] = fmaxf(a1, aN);
    }
    float amin = fmaxf(fmaxf(0.F, mins[0]), fmaxf(mins[1], mins[2]));
    float amax = fminf(fminf(1.F, maxs[0]), fminf(maxs[1], maxs[2]));
    if (rc_float_sup_eq(amin, amax)) return 0.F;

    /* plane index range per axis, Projector.cu:87-120 (truncating casts) */
    int lo_i[3], hi_i[3];
    for (int a = 0; a < 3; ++a) {
        float at_hi = d[a] > 0 ? amax : amin; /* alpha giving the max index */
        float at_lo = d[a] > 0 ? amin : amax;
        float up = (half[a] + s[a]) + at_hi * d[a];
        int mx = imax(0, imin(n[a] - 1, (int)up));
        float dn = (half[a] - s[a]) - at_lo * d[a];
        int mn = imax(0, imin(mx, n[a] - (int)dn));
        lo_i[a] = mn;
        hi_i[a] = mx;
    }

    /* alpha list, Projector.cu:122-201: x and y lists hold (max-min+1)
     * entries, the z list only 1 + max(0, (max-min)-2) (the count is short by
     * two, :182); every entry not written keeps the fill value 1.0. */
    unsigned total = (unsigned)(hi_i[0] - lo_i[0]) + (unsigned)(hi_i[1] - lo_i[1]) +
                     (unsigned)(hi_i[2] - lo_i[2]) + 3u;
    if (total > 4096u) total = 4096u; /* the reference has no guard; sizes here stay < 2000 */
    for (unsigned i = 0; i < total; ++i) alphas[i] = 1.0F;
    unsigned start = 0;
    for (int a = 0; a < 3; ++a) {
        int span = hi_i[a] - lo_i[a];
        unsigned count = (a < 2) ? (unsigned)span + 1u : (span >= 2 ? (unsigned)(span - 1) : 1u);
        if (fabsf(d[a]) > tol) {
            float step = 1.F / d[a];
            float first_plane = (float)(d[a] > 0 ? lo_i[a] : hi_i[a]);
            unsigned at = start;
            if (at < total) alphas[at] = step * ((-half[a] - s[a]) + first_plane);
            for (unsigned k = 1; k < count && at + k < total; ++k)
                alphas[at + k] = alphas[at + k - 1] + fabsf(step);
        }
        start += (a < 2) ? (unsigned)span + 1u : 0u;
    }
    if (ref_sort) selection_sort(alphas, total);
    else qsort(alphas, total, sizeof(float), cmp_float);

    /* midpoint lookup, Projector.cu:345-371: centre in double, truncation */
    float acc = 0.F, wsum = 0.F;
    const float base[3] = {half[0] + s[0], half[1] + s[1], half[2] + s[2]};
    for (unsigned i = 0; i + 1 < total; ++i) {
        double c = (double)(alphas[i + 1] + alphas[i]) / 2.0;
        int p[3];
        for (int a = 0; a < 3; ++a) p[a] = (int)((double)base[a] + c * (double)d[a]);
        float w = alphas[i + 1] - alphas[i];
        if (p[0] >= 0 && p[0] < n[0] && p[1] >= 0 && p[1] < n[1] && p[2] >= 0 && p[2] < n[2] &&
            w > tol) {
            size_t idx = ((size_t)p[2] * (size_t)n[1] + (size_t)p[1]) * (size_t)n[0] + (size_t)p[0];
            wsum += w;
            acc += w * vol[idx];
        }
    }
    return wsum > tol ? acc / wsum : 0.F;
}

static float rc_forward_ray(const kvo_geom *g, const float *vol, int view, int u, int v,
                            float *alphas) {
    return rc_forward_ray_sorted(g, vol, view, u, v, alphas, 0);
}

void kvo_rc_forward(const kvo_geom *g, const float *vol, float *proj) {
    const long long per_view = (long long)g->nu * g->nv;
    const long long nrays = per_view * g->n_views;
#pragma omp parallel
    {
        float *alphas = (float *)malloc(4096 * sizeof(float));
#pragma omp for schedule(dynamic, 256)
        for (long long r = 0; r < nrays; ++r) {
            int view = (int)(r / per_view);
            long long rem = r % per_view;
            int v = (int)(rem / g->nu), u = (int)(rem % g->nu);
            proj[r] = rc_forward_ray(g, vol, view, u, v, alphas);
        }
        free(alphas);
    }
}

/* Forward of a sampled subset of rays (ray indices into the projection
 * stack); used for CPU timing on large geometries. */
void kvo_rc_forward_rays(const kvo_geom *g, const float *vol, const int64_t *rays, int64_t n,
                         float *out) {
    const long long per_view = (long long)g->nu * g->nv;
#pragma omp parallel
    {
        float *alphas = (float *)malloc(4096 * sizeof(float));
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            long long r = rays[i];
            int view = (int)(r / per_view);
            long long rem = r % per_view;
            out[i] = rc_forward_ray(g, vol, view, (int)(rem % g->nu), (int)(rem / g->nu), alphas);
        }
        free(alphas);
    }
}

/* The same, ordering each ray's list with the reference's selection sort:
 * the reference's own per-ray cost, for timing its CPU path. */
void kvo_rc_forward_rays_refcost(const kvo_geom *g, const float *vol, const int64_t *rays, int64_t n,
                                 float *out) {
    const long long per_view = (long long)g->nu * g->nv;
#pragma omp parallel
    {
        float *alphas = (float *)malloc(4096 * sizeof(float));
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < n; ++i) {
            long long r = rays[i];
            long long rem = r % per_view;
            out[i] = rc_forward_ray_sorted(g, vol, (int)(r / per_view), (int)(rem % g->nu),
                                           (int)(rem / g->nu), alphas, 1);
        }
        free(alphas);
    }
}

/* One voxel of the RC backprojector, Projector.cu:387-776. */
static float rc_back_voxel(const kvo_geom *g, const float *proj, int x, int y, int z) {
    const float tol = 0.000000000000000000000001F; /* 1e-24, Projector.cu:416 */
    const int nu = g->nu, nv = g->nv;
    const int semi = 5; /* 11x11 window, Projector.cu:470 */
    float vf[3];
    vf[0] = (float)x - (float)g->nx / 2.F;
    vf[1] = (float)y - (float)g->ny / 2.F;
    vf[2] = (float)z - (float)g->nz / 2.F;
    float acc = 0.F, wsum = 0.F;
    for (int view = 0; view < g->n_views; ++view) {
        const float *sp = g->src + 3 * view, *op = g->det_origin + 3 * view;
        float s[3] = {sp[0] / g->dx, sp[1] / g->dy, sp[2] / g->dz};
        float o[3] = {op[0] / g->dx, op[1] / g->dy, op[2] / g->dz};
        float ex = (op[0] + (float)nu * g->du) / g->dx;
        float ey = (op[1] + (float)nv * g->dv) / g->dy;
        /* voxel-centre ray hits the detector plane, :473-492 */
        float c[3] = {vf[0] + 0.5F, vf[1] + 0.5F, vf[2] + 0.5F};
        float r[3] = {c[0] - s[0], c[1] - s[1], c[2] - s[2]};
        float az = fabsf(r[2]) > tol ? (o[2] - s[2]) / r[2] : 0.F;
        float hx = s[0] + r[0] * az, hy = s[1] + r[1] * az;
        float mx = (float)semi * g->du / g->dx, my = (float)semi * g->dv / g->dy;
        if (!(hx > o[0] - mx && hx < ex + mx && hy > o[1] - my && hy < ey + my)) continue;

        /* 11x11 window clamped to the detector, :607-646 */
        int px = (int)((hx - o[0]) * g->dx / g->du);
        int py = (int)((hy - o[1]) * g->dy / g->dv);
        int w0[2] = {px - semi, py - semi}, w1[2] = {px + semi, py + semi};
        const int lim[2] = {nu, nv};
        for (int a = 0; a < 2; ++a) {
            if (w0[a] < 0) w0[a] = 0; else if (w0[a] >= lim[a]) w0[a] = lim[a] - 1;
            if (w1[a] < 0) w1[a] = 0; else if (w1[a] >= lim[a]) w1[a] = lim[a] - 1;
        }
        /* pixel rays clipped against this voxel, :647-730 */
        const float *pv = proj + (size_t)view * (size_t)nu * (size_t)nv;
        float rz = op[2] / g->dz - s[2];
        float a1z = fabsf(rz) > tol ? (vf[2] - s[2]) / rz : 0.F;
        float a2z = fabsf(rz) > tol ? (vf[2] + 1.F - s[2]) / rz : 0.F;
        for (int qy = w0[1]; qy <= w1[1]; ++qy) {
            float ry = (op[1] + ((float)qy + 0.5F) * g->dv) / g->dy - s[1];
            float a1y = fabsf(ry) > tol ? (vf[1] - s[1]) / ry : 0.F;
            float a2y = fabsf(ry) > tol ? (vf[1] + 1.F - s[1]) / ry : 0.F;
            for (int qx = w0[0]; qx <= w1[0]; ++qx) {
                float rx = (op[0] + ((float)qx + 0.5F) * g->du) / g->dx - s[0];
                float a1x = fabsf(rx) > tol ? (vf[0] - s[0]) / rx : 0.F;
                float a2x = fabsf(rx) > tol ? (vf[0] + 1.F - s[0]) / rx : 0.F;
                float lo = fmaxf(fmaxf(0.F, fminf(a1x, a2x)), fmaxf(fminf(a1y, a2y), fminf(a1z, a2z)));
                float hi = fminf(fminf(1.F, fmaxf(a1x, a2x)), fminf(fmaxf(a1y, a2y), fmaxf(a1z, a2z)));
                if (rc_float_sup_eq(hi, lo)) {
                    float w = hi - lo;
                    if (w > tol) {
                        wsum += w;
                        acc += w * pv[(size_t)qy * nu + qx];
                    }
                }
            }
        }
    }
    return wsum > tol ? acc / wsum : 0.F;
}

void kvo_rc_back(const kvo_geom *g, const float *proj, float *vol) {
    const long long plane = (long long)g->nx * g->ny;
    const long long nvox = plane * g->nz;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < nvox; ++i) {
        int z = (int)(i / plane);
        long long rem = i % plane;
        vol[i] = rc_back_voxel(g, proj, (int)(rem % g->nx), (int)(rem / g->nx), z);
    }
}

/* Backprojection of a sampled subset of voxels (for CPU timing). */
void kvo_rc_back_voxels(const kvo_geom *g, const float *proj, const int64_t *voxels, int64_t n,
                        float *out) {
    const long long plane = (long long)g->nx * g->ny;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        long long v = voxels[i];
        long long rem = v % plane;
        out[i] = rc_back_voxel(g, proj, (int)(rem % g->nx), (int)(rem / g->nx), (int)(v / plane));
    }
}

/* AlmostEqualRelative(q, 0.f) of commons/Maths.h:25-34 holds only for q == 0. */
static int almost_equal_relative(float a, float b) {
    float diff = fabsf(a - b);
    float fa = fabsf(a), fb = fabsf(b);
    float scaled = 1.1920928955078125e-07F * (fa > fb ? fa : fb);
    return diff <= scaled;
}

/* The host loops of one recons::MLEM iteration on a sample of indices, as
 * the reference runs them (serial): the ratio q <- relax * p / q where
 * q != 0 (Reconstructors.h:207-213) over the sampled rays, and the update
 * x <- x * b (Reconstructors.h:238-241) over the sampled voxels. */
void kvo_rc_mlem_host_loops(const float *p, float *q, const int64_t *rays, int64_t n_rays, float *x,
                            const float *b, const int64_t *voxels, int64_t n_vox, float relax) {
    for (int64_t i = 0; i < n_rays; ++i) {
        const int64_t r = rays[i];
        if (!almost_equal_relative(q[r], 0.F)) q[r] = relax * (p[r] / q[r]);
    }
    for (int64_t i = 0; i < n_vox; ++i) {
        const int64_t j = voxels[i];
        x[j] *= b[j];
    }
}

/* recons::MLEM, Reconstructors.h:182-242; x updated in place. */
void kvo_rc_mlem(const kvo_geom *g, const float *p, float *x, int iters, float relax) {
    size_t np = (size_t)g->nu * g->nv * g->n_views, nvox = (size_t)g->nx * g->ny * g->nz;
    float *q = (float *)malloc(np * sizeof(float));
    float *b = (float *)malloc(nvox * sizeof(float));
    for (int it = 0; it < iters; ++it) {
        kvo_rc_forward(g, x, q);
        for (size_t i = 0; i < np; ++i)
            if (!almost_equal_relative(q[i], 0.F)) q[i] = relax * (p[i] / q[i]);
        kvo_rc_back(g, q, b);
        for (size_t j = 0; j < nvox; ++j) x[j] *= b[j];
    }
    free(q);
    free(b);
}

/* recons::ART, Reconstructors.h:65-122; x updated in place. */
void kvo_rc_art(const kvo_geom *g, const float *p, float *x, int iters, float relax) {
    size_t np = (size_t)g->nu * g->nv * g->n_views, nvox = (size_t)g->nx * g->ny * g->nz;
    float *q = (float *)malloc(np * sizeof(float));
    float *b = (float *)malloc(nvox * sizeof(float));
    for (int it = 0; it < iters; ++it) {
        kvo_rc_forward(g, x, q);
        for (size_t i = 0; i < np; ++i) q[i] = relax * (p[i] - q[i]);
        kvo_rc_back(g, q, b);
        for (size_t j = 0; j < nvox; ++j) x[j] += b[j];
    }
    free(q);
    free(b);
}

/* ---- shift-and-add ---------------------------------------------------- */

/* Integer row shift of view i for slice k.  rule 0 (RC) is the reference's
 * literal rule, Reconstructors.h:287-331: zF is the fulcrum height as given,
 * z_k the voxel-corner z of slice k in the volume-centred frame built as in
 * TomoVolume::UpdatePositions (float accumulation from -0.5*nz*dz), and the
 * shift is divided by the VOXEL y spacing.  rule 1 (EXACT) measures heights
 * from the detector plane at the slice centre and shifts in detector pixels:
 * t = round(y_src * (mZ - mF) / dv).  Returns -1 on the reference's error
 * conditions (fewer than 2 slices or views, fulcrum or a slice at the
 * source height). */
int kvo_saa_shifts(const kvo_geom *g, int rule, int32_t *shifts /* [nz][n_views] */) {
    if (g->nz <= 1 || g->n_views <= 1) return -1;
    float src_z = 0.F, det_z = 0.F;
    for (int i = 0; i < g->n_views; ++i) src_z += g->src[3 * i + 2];
    src_z /= (float)g->n_views;
    double acc = 0.0;
    for (int i = 0; i < g->n_views; ++i) acc += g->det_origin[3 * i + 2];
    det_z = (float)acc / (float)g->n_views;
    if (rule == 0) {
        float sid = fabsf(det_z - src_z);
        float zf = g->fulcrum_z;
        if (almost_equal_relative(zf, sid)) return -1;
        float mf = sid / (sid - zf);
        float wz = (float)g->nz * g->dz;
        float z = (float)(-0.5 * (double)wz);
        for (int k = 0; k < g->nz; ++k) {
            if (k > 0) z = z + g->dz;
            if (almost_equal_relative(z, sid)) return -1;
            float mz = sid / (sid - z);
            float coeff = mz - mf;
            for (int i = 0; i < g->n_views; ++i) {
                float t = g->src[3 * i + 1] * coeff;
                shifts[(size_t)k * g->n_views + i] = (int32_t)(t / g->dy);
            }
        }
    } else {
        double sid = (double)src_z - (double)det_z;
        double hf = (double)g->fulcrum_z - (double)det_z;
        if (fabs(sid - hf) < 1e-9 * fabs(sid)) return -1;
        double mf = sid / (sid - hf);
        for (int k = 0; k < g->nz; ++k) {
            double zc = -0.5 * (double)g->nz * g->dz + ((double)k + 0.5) * g->dz;
            double hz = zc - (double)det_z;
            if (fabs(sid - hz) < 1e-9 * fabs(sid)) return -1;
            double mz = sid / (sid - hz);
            for (int i = 0; i < g->n_views; ++i) {
                double t = (double)g->src[3 * i + 1] * (mz - mf) / (double)g->dv;
                shifts[(size_t)k * g->n_views + i] = (int32_t)lround(t);
            }
        }
    }
    return 0;
}

/* out[k][v][u] = sum_i (1/P) * in[i][v + t_ki][u] (zero outside the ROI),
 * summed in double and rounded to float (vtkImageWeightedSum). */
void kvo_saa(const kvo_geom *g, const int32_t *shifts, const float *proj, float *out) {
    const int nu = g->nu, nv = g->nv, P = g->n_views;
    const double w = 1. / (double)P;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < g->nz; ++k)
        for (int v = 0; v < nv; ++v)
            for (int u = 0; u < nu; ++u) {
                double s = 0.0;
                for (int i = 0; i < P; ++i) {
                    int r = v + shifts[(size_t)k * P + i];
                    if (r >= 0 && r < nv) s += w * (double)proj[((size_t)i * nv + r) * nu + u];
                }
                out[((size_t)k * nv + v) * nu + u] = (float)s;
            }
}

/* ======================================================================
 * EXACT family, FP64 Siddon
 * ====================================================================== */

typedef struct {
    double s[3], d[3], len, amin, amax;
    double b0[3], sp[3];
    int n[3];
} exact_ray;

/* Returns 0 if the ray misses the box. */
static int exact_ray_setup(const kvo_geom *g, int view, double pu, double pv, exact_ray *r) {
    const float *sp = g->src + 3 * view, *op = g->det_origin + 3 * view;
    r->n[0] = g->nx; r->n[1] = g->ny; r->n[2] = g->nz;
    r->sp[0] = g->dx; r->sp[1] = g->dy; r->sp[2] = g->dz;
    double p[3] = {(double)op[0] + pu * g->du, (double)op[1] + pv * g->dv, (double)op[2]};
    for (int a = 0; a < 3; ++a) {
        r->s[a] = sp[a];
        r->d[a] = p[a] - r->s[a];
        r->b0[a] = -0.5 * r->n[a] * r->sp[a];
    }
    r->len = sqrt(r->d[0] * r->d[0] + r->d[1] * r->d[1] + r->d[2] * r->d[2]);
    double lo = 0.0, hi = 1.0;
    for (int a = 0; a < 3; ++a) {
        double b1 = r->b0[a] + r->n[a] * r->sp[a];
        if (r->d[a] == 0.0) {
            if (r->s[a] < r->b0[a] || r->s[a] >= b1) return 0;
            continue;
        }
        double t0 = (r->b0[a] - r->s[a]) / r->d[a], t1 = (b1 - r->s[a]) / r->d[a];
        if (t0 > t1) { double t = t0; t0 = t1; t1 = t; }
        if (t0 > lo) lo = t0;
        if (t1 < hi) hi = t1;
    }
    r->amin = lo;
    r->amax = hi;
    return hi > lo;
}

/* Walks the ray through the voxels (Jacobs' incremental Siddon with the
 * crossing alphas recomputed from plane indices).  Calls visit(idx, w) with
 * w the intersection length in mm. */
#define EXACT_WALK(r, BODY)                                                                   \
    do {                                                                                      \
        double alpha = (r).amin;                                                              \
        double mid0[3];                                                                       \
        int idx3[3], step3[3];                                                                \
        double next3[3], inc3[3];                                                             \
        /* voxel containing the entry point: classify a point slightly inside */              \
        double probe = (r).amin + 1e-9 * ((r).amax - (r).amin);                               \
        for (int a = 0; a < 3; ++a) {                                                         \
            mid0[a] = (r).s[a] + probe * (r).d[a];                                            \
            idx3[a] = (int)floor((mid0[a] - (r).b0[a]) / (r).sp[a]);                          \
            if (idx3[a] < 0) idx3[a] = 0;                                                     \
            if (idx3[a] >= (r).n[a]) idx3[a] = (r).n[a] - 1;                                  \
            if ((r).d[a] > 0) {                                                               \
                step3[a] = 1;                                                                 \
                next3[a] = ((r).b0[a] + (idx3[a] + 1) * (r).sp[a] - (r).s[a]) / (r).d[a];     \
                inc3[a] = (r).sp[a] / (r).d[a];                                               \
            } else if ((r).d[a] < 0) {                                                        \
                step3[a] = -1;                                                                \
                next3[a] = ((r).b0[a] + idx3[a] * (r).sp[a] - (r).s[a]) / (r).d[a];           \
                inc3[a] = -(r).sp[a] / (r).d[a];                                              \
            } else {                                                                          \
                step3[a] = 0;                                                                 \
                next3[a] = INFINITY;                                                          \
                inc3[a] = 0;                                                                  \
            }                                                                                 \
        }                                                                                     \
        while (alpha < (r).amax) {                                                            \
            int m = 0;                                                                        \
            if (next3[1] < next3[m]) m = 1;                                                   \
            if (next3[2] < next3[m]) m = 2;                                                   \
            double an = next3[m] < (r).amax ? next3[m] : (r).amax;                            \
            double w_mm = (an - alpha) * (r).len;                                             \
            size_t vidx = ((size_t)idx3[2] * (r).n[1] + idx3[1]) * (r).n[0] + idx3[0];        \
            if (w_mm > 0) { BODY }                                                            \
            alpha = an;                                                                       \
            if (an >= (r).amax) break;                                                        \
            idx3[m] += step3[m];                                                              \
            if (idx3[m] < 0 || idx3[m] >= (r).n[m]) break;                                    \
            int pl = step3[m] > 0 ? idx3[m] + 1 : idx3[m];                                    \
            next3[m] = ((r).b0[m] + pl * (r).sp[m] - (r).s[m]) / (r).d[m];                    \
            (void)inc3;                                                                       \
        }                                                                                     \
    } while (0)

static double exact_forward_ray(const kvo_geom *g, const double *vol, int view, int u, int v) {
    exact_ray r;
    if (!exact_ray_setup(g, view, u + 0.5, v + 0.5, &r)) return 0.0;
    double acc = 0.0;
    EXACT_WALK(r, { acc += w_mm * vol[vidx]; });
    return acc;
}

void kvo_exact_forward(const kvo_geom *g, const double *vol, double *proj) {
    const long long per_view = (long long)g->nu * g->nv;
    const long long nrays = per_view * g->n_views;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long r = 0; r < nrays; ++r) {
        int view = (int)(r / per_view);
        long long rem = r % per_view;
        proj[r] = exact_forward_ray(g, vol, view, (int)(rem % g->nu), (int)(rem / g->nu));
    }
}

void kvo_exact_forward_rays(const kvo_geom *g, const double *vol, const int64_t *rays, int64_t n,
                            double *out) {
    const long long per_view = (long long)g->nu * g->nv;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        long long r = rays[i];
        long long rem = r % per_view;
        out[i] = exact_forward_ray(g, vol, (int)(r / per_view), (int)(rem % g->nu), (int)(rem / g->nu));
    }
}

/* Total intersection length of each ray with the volume box (A 1). */
void kvo_exact_ray_lengths(const kvo_geom *g, double *out) {
    const long long per_view = (long long)g->nu * g->nv;
    const long long nrays = per_view * g->n_views;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nrays; ++i) {
        exact_ray r;
        int view = (int)(i / per_view);
        long long rem = i % per_view;
        out[i] = exact_ray_setup(g, view, (int)(rem % g->nu) + 0.5, (int)(rem / g->nu) + 0.5, &r)
                     ? (r.amax - r.amin) * r.len : 0.0;
    }
}

/* Transpose: scatter each ray's value times its intersection lengths.
 * Views are split across threads, each with a private accumulator. */
void kvo_exact_back(const kvo_geom *g, const double *proj, double *vol) {
    const size_t nvox = (size_t)g->nx * g->ny * g->nz;
    const long long per_view = (long long)g->nu * g->nv;
    memset(vol, 0, nvox * sizeof(double));
    int nt = kvo_num_threads();
    if (nt > g->n_views) nt = g->n_views;
    if (nt < 1) nt = 1;
    double *priv = (double *)calloc((size_t)nt * nvox, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
    for (int view = 0; view < g->n_views; ++view) {
#ifdef _OPENMP
        double *acc = priv + (size_t)omp_get_thread_num() * nvox;
#else
        double *acc = priv;
#endif
        for (long long rem = 0; rem < per_view; ++rem) {
            double val = proj[(size_t)view * per_view + rem];
            if (val == 0.0) continue;
            exact_ray r;
            if (!exact_ray_setup(g, view, (int)(rem % g->nu) + 0.5, (int)(rem / g->nu) + 0.5, &r))
                continue;
            EXACT_WALK(r, { acc[vidx] += w_mm * val; });
        }
    }
    for (int t = 0; t < nt; ++t)
        for (size_t j = 0; j < nvox; ++j) vol[j] += priv[(size_t)t * nvox + j];
    free(priv);
}

/* Transpose restricted to a subset of rays: vol += sum_r values[r] * (row r
 * of A), scattered with atomic adds (for timing the CPU path on a sample). */
void kvo_exact_back_rays(const kvo_geom *g, const double *values, const int64_t *rays, int64_t n,
                         double *vol) {
    const long long per_view = (long long)g->nu * g->nv;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
        long long r = rays[i];
        long long rem = r % per_view;
        exact_ray ray;
        if (!exact_ray_setup(g, (int)(r / per_view), (int)(rem % g->nu) + 0.5, (int)(rem / g->nu) + 0.5, &ray))
            continue;
        const double val = values[i];
        EXACT_WALK(ray, { _Pragma("omp atomic") vol[vidx] += w_mm * val; });
    }
}

/* EXACT MLEM in FP64: x <- x * A^T(relax p / A x) / A^T 1. */
void kvo_exact_mlem(const kvo_geom *g, const double *p, double *x, int iters, double relax) {
    size_t np = (size_t)g->nu * g->nv * g->n_views, nvox = (size_t)g->nx * g->ny * g->nz;
    double *q = (double *)malloc(np * sizeof(double));
    double *b = (double *)malloc(nvox * sizeof(double));
    double *sens = (double *)malloc(nvox * sizeof(double));
    for (size_t i = 0; i < np; ++i) q[i] = 1.0;
    kvo_exact_back(g, q, sens);
    for (int it = 0; it < iters; ++it) {
        kvo_exact_forward(g, x, q);
        for (size_t i = 0; i < np; ++i) q[i] = q[i] > 0.0 ? relax * p[i] / q[i] : 0.0;
        kvo_exact_back(g, q, b);
        for (size_t j = 0; j < nvox; ++j)
            if (sens[j] > 0.0) x[j] = x[j] * b[j] / sens[j];
    }
    free(q);
    free(b);
    free(sens);
}

/* EXACT SART in FP64: x <- x + relax * C A^T(R (p - A x)). */
void kvo_exact_sart(const kvo_geom *g, const double *p, double *x, int iters, double relax) {
    size_t np = (size_t)g->nu * g->nv * g->n_views, nvox = (size_t)g->nx * g->ny * g->nz;
    double *q = (double *)malloc(np * sizeof(double));
    double *rows = (double *)malloc(np * sizeof(double));
    double *b = (double *)malloc(nvox * sizeof(double));
    double *cols = (double *)malloc(nvox * sizeof(double));
    kvo_exact_ray_lengths(g, rows);
    for (size_t i = 0; i < np; ++i) q[i] = 1.0;
    kvo_exact_back(g, q, cols);
    for (int it = 0; it < iters; ++it) {
        kvo_exact_forward(g, x, q);
        for (size_t i = 0; i < np; ++i) q[i] = rows[i] > 0.0 ? (p[i] - q[i]) / rows[i] : 0.0;
        kvo_exact_back(g, q, b);
        for (size_t j = 0; j < nvox; ++j)
            if (cols[j] > 0.0) x[j] += relax * b[j] / cols[j];
    }
    free(q);
    free(rows);
    free(b);
    free(cols);
}

/* ======================================================================
 * Phantom: sum of ellipsoids sampled at voxel centres
 * ====================================================================== */

/* params: n x 16 floats = centre[3], semi-axes[3], R[9] (row-major, local =
 * R (q - c)), density.  Float arithmetic in a fixed order; the GPU rasteriser
 * uses the same order. */
void kvo_phantom(int nx, int ny, int nz, float dx, float dy, float dz, const float *params, int n,
                 float *vol) {
    const long long plane = (long long)nx * ny;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < plane * nz; ++i) {
        int z = (int)(i / plane);
        long long rem = i % plane;
        int y = (int)(rem / nx), x = (int)(rem % nx);
        float q[3] = {((float)x + 0.5F) * dx - 0.5F * (float)nx * dx,
                      ((float)y + 0.5F) * dy - 0.5F * (float)ny * dy,
                      ((float)z + 0.5F) * dz - 0.5F * (float)nz * dz};
        float val = 0.F;
        for (int e = 0; e < n; ++e) {
            const float *p = params + 16 * e;
            float r0 = q[0] - p[0], r1 = q[1] - p[1], r2 = q[2] - p[2];
            float l0 = (p[6] * r0 + p[7] * r1) + p[8] * r2;
            float l1 = (p[9] * r0 + p[10] * r1) + p[11] * r2;
            float l2 = (p[12] * r0 + p[13] * r1) + p[14] * r2;
            float t0 = l0 / p[3], t1 = l1 / p[4], t2 = l2 / p[5];
            float s = (t0 * t0 + t1 * t1) + t2 * t2;
            if (s <= 1.F) val += p[15];
        }
        vol[i] = val;
    }
}
