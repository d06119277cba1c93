/*
 * ref_driver.cpp -- host driver for the reference kernels compiled on the CPU
 * (TEST INFRASTRUCTURE; built by oracle/build_ref.sh into oracle/_ref/).
 *
 * Exposes the reference's own CudaPerformProjection (Projector.cu:227-372)
 * and CudaPerformBackProjection (Projector.cu:376-785) over a whole geometry,
 * launched the way Projector::PerformProjection / PerformBackProjection do
 * (Projector.cu:917-954, 1082-1125): per-view float3 detector origins and
 * source positions, pixel spacing as float2, the volume origin (unused by the
 * kernels).  Rays that miss the volume are not run -- the reference returns an
 * undefined value there (Projector.cu:79-85) -- and are written as 0, the
 * value Projector.cu:273 stores before the ray is traced.
 */
#include "ref_shim.h"

#include <cstdint>
#include <vector>

thread_local dim3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 threadIdx;

#include "ref_kernels_cpu.inc"

namespace {
struct Geom {
    int32_t nx, ny, nz;
    float dx, dy, dz;
    int32_t n_views;
    int32_t nu, nv;
    float du, dv;
    const float *src;
    const float *det_origin;
    float fulcrum_z;
};

/* Box test of FindProjectionAlphas_d (Projector.cu:47-85), used only to skip
 * the rays on which the reference kernel has no defined result. */
bool ray_hits(const Geom &g, int view, int u, int v) {
    const float tol = 0.000001F;
    const float sp[3] = {g.dx, g.dy, g.dz};
    const int n[3] = {g.nx, g.ny, g.nz};
    const float *s0 = g.src + 3 * view, *o = g.det_origin + 3 * view;
    float s[3], p[3], d[3];
    for (int a = 0; a < 3; ++a) s[a] = s0[a] / sp[a];
    p[0] = (o[0] + ((float)u + 0.5F) * g.du) / g.dx;
    p[1] = (o[1] + ((float)v + 0.5F) * g.dv) / g.dy;
    p[2] = o[2] / g.dz;
    float mins[3], maxs[3];
    for (int a = 0; a < 3; ++a) {
        d[a] = p[a] - s[a];
        float h = (float)n[a] / 2.F;
        float a1 = std::fabs(d[a]) > tol ? (-h - s[a]) / d[a] : 0.F;
        float an = std::fabs(d[a]) > tol ? (h - s[a]) / d[a] : 0.F;
        mins[a] = std::fmin(a1, an);
        maxs[a] = std::fmax(a1, an);
    }
    float lo = std::fmax(std::fmax(0.F, mins[0]), std::fmax(mins[1], mins[2]));
    float hi = std::fmin(std::fmin(1.F, maxs[0]), std::fmin(maxs[1], maxs[2]));
    float diff = lo - hi;
    bool sup_eq = lo > hi || (diff < 0.0000001F && diff > -0.0000001F);
    return !sup_eq;
}

void views(const Geom &g, std::vector<float3> &org, std::vector<float3> &src) {
    org.resize(g.n_views);
    src.resize(g.n_views);
    for (int i = 0; i < g.n_views; ++i) {
        org[i] = {g.det_origin[3 * i], g.det_origin[3 * i + 1], g.det_origin[3 * i + 2]};
        src[i] = {g.src[3 * i], g.src[3 * i + 1], g.src[3 * i + 2]};
    }
}
}  // namespace

extern "C" void kvref_forward(const Geom *g, const float *vol, float *proj) {
    std::vector<float3> org, src;
    views(*g, org, src);
    dim3 vdim(g->nx, g->ny, g->nz), pdim(g->nu, g->nv, g->n_views);
    float3 vorg{0.F, 0.F, 0.F}, vsp{g->dx, g->dy, g->dz};
    float2 psp{g->du, g->dv};
    const long long per_view = (long long)g->nu * g->nv, n = per_view * g->n_views;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long r = 0; r < n; ++r) {
        int view = (int)(r / per_view);
        int v = (int)((r % per_view) / g->nu), u = (int)(r % g->nu);
        if (!ray_hits(*g, view, u, v)) {
            proj[r] = 0.F;
            continue;
        }
        blockDim = dim3(1, 1, 1);
        threadIdx = dim3(0, 0, 0);
        blockIdx = dim3(u, v, view);
        CudaPerformProjection(vol, vdim, vorg, vsp, proj, pdim, psp, org.data(), src.data());
    }
}

extern "C" void kvref_back(const Geom *g, const float *proj, float *vol) {
    std::vector<float3> org, src;
    views(*g, org, src);
    dim3 vdim(g->nx, g->ny, g->nz), pdim(g->nu, g->nv, g->n_views);
    float3 vorg{0.F, 0.F, 0.F}, vsp{g->dx, g->dy, g->dz};
    float2 psp{g->du, g->dv};
    const long long plane = (long long)g->nx * g->ny, n = plane * g->nz;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < n; ++i) {
        blockDim = dim3(1, 1, 1);
        threadIdx = dim3(0, 0, 0);
        blockIdx = dim3((unsigned)(i % g->nx), (unsigned)((i % plane) / g->nx), (unsigned)(i / plane));
        CudaPerformBackProjection(proj, vdim, vorg, vsp, vol, pdim, psp, org.data(), src.data());
    }
}

/* The reference's kernels on a sample: rays (indices into the projection
 * stack) and voxels (indices into the volume), written into full-size
 * buffers at those indices.  Used to time the reference's own CPU path on a
 * bounded sample of a large workload. */
extern "C" void kvref_forward_rays(const Geom *g, const float *vol, const int64_t *rays, int64_t n, float *proj) {
    std::vector<float3> org, src;
    views(*g, org, src);
    dim3 vdim(g->nx, g->ny, g->nz), pdim(g->nu, g->nv, g->n_views);
    float3 vorg{0.F, 0.F, 0.F}, vsp{g->dx, g->dy, g->dz};
    float2 psp{g->du, g->dv};
    const long long per_view = (long long)g->nu * g->nv;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
        const long long r = rays[i];
        int view = (int)(r / per_view);
        int v = (int)((r % per_view) / g->nu), u = (int)(r % g->nu);
        if (!ray_hits(*g, view, u, v)) {
            proj[r] = 0.F;
            continue;
        }
        blockDim = dim3(1, 1, 1);
        threadIdx = dim3(0, 0, 0);
        blockIdx = dim3(u, v, view);
        CudaPerformProjection(vol, vdim, vorg, vsp, proj, pdim, psp, org.data(), src.data());
    }
}

extern "C" void kvref_back_voxels(const Geom *g, const float *proj, const int64_t *voxels, int64_t n, float *vol) {
    std::vector<float3> org, src;
    views(*g, org, src);
    dim3 vdim(g->nx, g->ny, g->nz), pdim(g->nu, g->nv, g->n_views);
    float3 vorg{0.F, 0.F, 0.F}, vsp{g->dx, g->dy, g->dz};
    float2 psp{g->du, g->dv};
    const long long plane = (long long)g->nx * g->ny;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
        const long long w = voxels[i];
        blockDim = dim3(1, 1, 1);
        threadIdx = dim3(0, 0, 0);
        blockIdx = dim3((unsigned)(w % g->nx), (unsigned)((w % plane) / g->nx), (unsigned)(w / plane));
        CudaPerformBackProjection(proj, vdim, vorg, vsp, vol, pdim, psp, org.data(), src.data());
    }
}
