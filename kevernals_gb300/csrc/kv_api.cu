// kv_api.cu -- the C ABI (include/kvtomo.h): contexts, plans, operators and
// the iterative drivers.  Host code only; the kernels live in kv_exact.cu,
// kv_rc.cu and kv_misc.cu.
#include "kv_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------

kv_status kv_fail(kv_ctx *ctx, kv_status s, const char *fmt, ...) {
    if (ctx != nullptr) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return s;
}

namespace {

bool stream_capturing(kv_ctx *ctx);

// Error bits that self-checking kernels leave in ctx->d_status (a bounded
// wait that gave up, a ray outside its staged box), read at the points where
// the call synchronises anyway, cleared, and returned as a status.
kv_status device_status(kv_ctx *ctx) {
    if (ctx->d_status == nullptr || stream_capturing(ctx)) return KV_OK;
    int h = 0;
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_status, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h == 0) return KV_OK;
    KV_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    return kv_fail(ctx, (h & 9) ? KV_ERR_TIMEOUT : KV_ERR_CUDA,
                   "a projector kernel stopped early (status bits 0x%x: 1 = a staged load did not arrive, "
                   "2/4 = a ray left its staged box, 8 = a staged detector patch did not arrive, "
                   "16 = a voxel tile's candidates left its staged patch)", h);
}

kv_status residual_from_red(kv_ctx *ctx, double *res, double *ll) {
    double h[3];
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_red, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    KV_TRY(device_status(ctx));
    if (res) *res = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    if (ll) *ll = h[2];
    return KV_OK;
}

template <typename T>
kv_status ensure(kv_ctx *ctx, T **p, size_t bytes) {
    if (*p == nullptr) KV_CHECK_CUDA(ctx, cudaMalloc((void **)p, bytes));
    return KV_OK;
}

// Resolves a caller float buffer to a device pointer: device memory is used
// as is; host memory goes through a plan workspace buffer (copied in when
// `copy_in`).
kv_status stage_in(kv_plan *plan, const float *user, kv_mem mem, float **staging, size_t n,
                   bool copy_in, float **dev) {
    if (mem == KV_MEM_DEVICE) {
        *dev = const_cast<float *>(user);
        return KV_OK;
    }
    KV_TRY(ensure(plan->ctx, staging, n * sizeof(float)));
    if (copy_in)
        KV_CHECK_CUDA(plan->ctx, cudaMemcpyAsync(*staging, user, n * sizeof(float), cudaMemcpyHostToDevice,
                                                 plan->ctx->stream));
    *dev = *staging;
    return KV_OK;
}

kv_status stage_out(kv_plan *plan, float *user, kv_mem mem, const float *dev, size_t n) {
    if (mem == KV_MEM_DEVICE) return KV_OK;
    KV_CHECK_CUDA(plan->ctx, cudaMemcpyAsync(user, dev, n * sizeof(float), cudaMemcpyDeviceToHost,
                                             plan->ctx->stream));
    KV_CHECK_CUDA(plan->ctx, cudaStreamSynchronize(plan->ctx->stream));
    return device_status(plan->ctx);
}

kv_status check_common(kv_plan *plan, const void *a, const void *b, kv_mem mem) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (a == nullptr || b == nullptr) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "null buffer");
    if (mem != KV_MEM_HOST && mem != KV_MEM_DEVICE) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "bad kv_mem");
    KV_CHECK_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
    return KV_OK;
}

kv_status ensure_sens(kv_plan *plan) {
    if (plan->sens_valid) return KV_OK;
    KV_TRY(ensure(plan->ctx, &plan->d_sens, plan->nvox * sizeof(double)));
    KV_TRY(exact_sensitivity_launch(plan, plan->d_sens));
    plan->sens_valid = true;
    return KV_OK;
}

// The geometry's values, beyond the sizes: positive finite spacings and
// pitches, a finite fulcrum, finite source and detector positions.
kv_status check_geometry_values(kv_ctx *ctx, const kv_geometry &g) {
    auto pos = [](float v) { return std::isfinite(v) && v > 0.f; };
    if (!pos(g.dx) || !pos(g.dy) || !pos(g.dz) || !pos(g.du) || !pos(g.dv))
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "spacings must be positive and finite");
    if (!std::isfinite(g.fulcrum_z)) return kv_fail(ctx, KV_ERR_NUMERIC, "non-finite fulcrum height");
    for (int i = 0; i < 3 * g.n_views; ++i)
        if (!std::isfinite(g.src[i]) || !std::isfinite(g.det_origin[i]))
            return kv_fail(ctx, KV_ERR_NUMERIC, "non-finite source / detector position");
    return KV_OK;
}

// A row shift (after the rule's own rounding or truncation) as an int32,
// limited to +-limit so that the conversion is defined.
constexpr int32_t kMaxShift = 1 << 30;
template <typename T>
int32_t stored_shift(T t, int32_t limit) {
    if (t >= (T)limit) return limit;
    if (t <= -(T)limit) return -limit;
    return (int32_t)t;
}

// Integer row shifts of shift-and-add, one per (slice, view).
// rule RC follows recons::ShiftAndAdd literally (Reconstructors.h:287-331);
// rule EXACT uses heights above the detector plane and detector pixels.
kv_status saa_shifts(kv_ctx *ctx, const kv_geometry &g, kv_family family, int32_t *sh) {
    const int P = g.n_views, nz = g.nz;
    if (nz <= 1) return kv_fail(ctx, KV_ERR_GEOMETRY, "shift-and-add needs at least 2 slices (got %d)", nz);
    if (P <= 1) return kv_fail(ctx, KV_ERR_GEOMETRY, "shift-and-add needs at least 2 projections (got %d)", P);
    if (g.nv <= 0) return kv_fail(ctx, KV_ERR_INVALID_ARG, "sizes must be positive");
    KV_TRY(check_geometry_values(ctx, g));
    // common source z (TomoTable: float mean) and detector z (double sum, float mean)
    float src_z = 0.f;
    for (int i = 0; i < P; ++i) src_z += g.src[3 * i + 2];
    src_z /= (float)P;
    double acc = 0.0;
    for (int i = 0; i < P; ++i) acc += g.det_origin[3 * i + 2];
    const float det_z = (float)acc / (float)P;
    auto almost_equal = [](float a, float b) {
        float d = std::fabs(a - b), fa = std::fabs(a), fb = std::fabs(b);
        return d <= 1.1920928955078125e-07f * (fa > fb ? fa : fb);
    };
    if (family == KV_FAMILY_RC) {
        const float sid = std::fabs(det_z - src_z);
        const float zf = g.fulcrum_z;
        if (almost_equal(zf, sid)) return kv_fail(ctx, KV_ERR_GEOMETRY, "fulcrum at the source height");
        const float mf = sid / (sid - zf);
        const float wz = (float)nz * g.dz;
        float z = (float)(-0.5 * (double)wz);
        for (int k = 0; k < nz; ++k) {
            if (k > 0) z = z + g.dz;
            if (almost_equal(z, sid)) return kv_fail(ctx, KV_ERR_GEOMETRY, "slice %d at the source height", k);
            const float coeff = sid / (sid - z) - mf;
            for (int i = 0; i < P; ++i) {
                const float t = g.src[3 * i + 1] * coeff;
                const float q = t / g.dy;
                if (std::isnan(q)) return kv_fail(ctx, KV_ERR_NUMERIC, "non-finite shift at slice %d", k);
                sh[(size_t)k * P + i] = stored_shift(std::trunc(q), kMaxShift);
            }
        }
    } else {
        const double sid = (double)src_z - (double)det_z;
        const double hf = (double)g.fulcrum_z - (double)det_z;
        if (std::fabs(sid - hf) < 1e-9 * std::fabs(sid)) return kv_fail(ctx, KV_ERR_GEOMETRY, "fulcrum at the source height");
        const double mf = sid / (sid - hf);
        for (int k = 0; k < nz; ++k) {
            const double hz = -0.5 * nz * (double)g.dz + (k + 0.5) * (double)g.dz - (double)det_z;
            if (std::fabs(sid - hz) < 1e-9 * std::fabs(sid)) return kv_fail(ctx, KV_ERR_GEOMETRY, "slice %d at the source height", k);
            const double mz = sid / (sid - hz);
            for (int i = 0; i < P; ++i) {
                const double q = (double)g.src[3 * i + 1] * (mz - mf) / (double)g.dv;
                if (std::isnan(q)) return kv_fail(ctx, KV_ERR_NUMERIC, "non-finite shift at slice %d", k);
                sh[(size_t)k * P + i] = stored_shift(std::round(q), kMaxShift);
            }
        }
    }
    return KV_OK;
}

// Host-buffer calls overlap their copies with the kernels on a second
// (non-blocking) stream of the context, in at most kOverlapChunks pieces.
constexpr int kOverlapChunks = 8;
// A projector pass over one view or slice takes ~10-20x as long as copying
// that view or slice at the host link's ~200 GB/s, so pieces may grow by
// this factor and each copy still hides behind the previous piece's kernels.
constexpr int kOverlapGrowth = 4;

// Piece boundaries of [0, total): sizes 1, g, g^2, ... (the last piece takes
// the rest), at most kOverlapChunks pieces.  Uploads use them in this order
// (the first piece's copy is the only one that nothing hides); downloads
// reversed (the last piece's copy is).  Few pieces keep the launches few.
std::vector<int> overlap_bounds(int total, bool shrinking) {
    std::vector<int> sizes;
    int left = total;
    for (long long sz = 1; left > 0; sz *= kOverlapGrowth) {
        const int take = (int)sizes.size() == kOverlapChunks - 1 ? left : (int)std::min<long long>(sz, left);
        sizes.push_back(take);
        left -= take;
    }
    if (shrinking) std::reverse(sizes.begin(), sizes.end());
    std::vector<int> b(1, 0);
    for (int v : sizes) b.push_back(b.back() + v);
    return b;
}

kv_status ensure_copy_stream(kv_ctx *ctx) {
    if (ctx->copy_stream == nullptr)
        KV_CHECK_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    while (ctx->copy_events.size() < 1 + 2 * kOverlapChunks) {
        cudaEvent_t e;
        KV_CHECK_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->copy_events.push_back(e);
    }
    return KV_OK;
}

// Runs launch(i0, n) on the context stream for the (shrinking) pieces of
// [0, total) and copies each piece's output (dev + i0 * stride, n * stride
// floats) to the same place in host memory on the copy stream as soon as
// that piece's kernels are done.  Events ev0 .. ev0 + kOverlapChunks - 1.
template <typename Launch>
kv_status pieces_to_host_body(kv_ctx *ctx, int total, size_t stride, const float *dev, float *host, int ev0,
                              Launch &launch) {
    cudaEvent_t *ev = ctx->copy_events.data() + ev0;
    const std::vector<int> b = overlap_bounds(total, true);
    const int np = (int)b.size() - 1;
    for (int c = 0; c < np; ++c) {
        KV_TRY(launch(b[c], b[c + 1] - b[c]));
        KV_CHECK_CUDA(ctx, cudaEventRecord(ev[c], ctx->stream));
    }
    for (int c = 0; c < np; ++c) {
        const size_t n = (size_t)(b[c + 1] - b[c]) * stride;
        KV_CHECK_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ev[c], 0));
        KV_CHECK_CUDA(ctx, cudaMemcpyAsync(host + b[c] * stride, dev + b[c] * stride, n * sizeof(float),
                                           cudaMemcpyDeviceToHost, ctx->copy_stream));
    }
    return KV_OK;
}

// Waits for both streams, so that no copy is in flight when the caller's
// buffers are handed back; returns the first error.
kv_status sync_both(kv_ctx *ctx, kv_status s) {
    cudaError_t e1 = cudaStreamSynchronize(ctx->copy_stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (s != KV_OK) return s;
    if (e1 != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "copy stream: %s", cudaGetErrorString(e1));
    if (e2 != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "stream: %s", cudaGetErrorString(e2));
    return device_status(ctx);
}

bool stream_capturing(kv_ctx *ctx) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(ctx->stream, &cs);
    return cs != cudaStreamCaptureStatusNone;
}

}  // namespace

// ---------------------------------------------------------------------------
// Library / context
// ---------------------------------------------------------------------------

extern "C" const char *kv_version(void) { return "kvtomo 0.1.0 (sm_103a)"; }

extern "C" const char *kv_status_string(kv_status s) {
    switch (s) {
    case KV_OK: return "ok";
    case KV_ERR_INVALID_ARG: return "invalid argument";
    case KV_ERR_GEOMETRY: return "geometry not supported";
    case KV_ERR_OOM: return "out of memory";
    case KV_ERR_CUDA: return "CUDA error";
    case KV_ERR_TIMEOUT: return "device wait timed out";
    case KV_ERR_NUMERIC: return "numeric error";
    case KV_ERR_UNSUPPORTED: return "unsupported";
    case KV_ERR_NO_DEVICE: return "no sm_103 device";
    }
    return "unknown status";
}

extern "C" kv_status kv_ctx_create(int device, kv_ctx **out) {
    if (out == nullptr) return KV_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return KV_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return KV_ERR_INVALID_ARG;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return KV_ERR_CUDA;
    if (!(prop.major == 10 && prop.minor == 3)) return KV_ERR_NO_DEVICE;
    kv_ctx *ctx = new (std::nothrow) kv_ctx;
    if (ctx == nullptr) return KV_ERR_OOM;
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void **)&ctx->d_red, 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaFree(ctx->d_red);
        cudaFree(ctx->d_status);
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
        delete ctx;
        return KV_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return KV_OK;
}

namespace {
void ctx_free(kv_ctx *ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (const kv_timing_rec &r : ctx->timing_recs) {
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (cudaEvent_t e : ctx->copy_events) cudaEventDestroy(e);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    cudaFree(ctx->d_red);
    cudaFree(ctx->d_status);
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}
}  // namespace

// Releases the caller's reference; the context lives on until its last plan
// is destroyed, so destroying a context before its plans is safe.
extern "C" kv_status kv_ctx_destroy(kv_ctx *ctx) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (ctx->released) return kv_fail(ctx, KV_ERR_INVALID_ARG, "context destroyed twice");
    ctx->released = true;
    if (ctx->plans == 0) ctx_free(ctx);
    return KV_OK;
}

extern "C" kv_status kv_ctx_set_stream(kv_ctx *ctx, void *stream) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    ctx->stream = (cudaStream_t)stream;   // NULL: the CUDA default stream
    return KV_OK;
}

extern "C" kv_status kv_sync(kv_ctx *ctx) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return device_status(ctx);
}

extern "C" const char *kv_ctx_last_error(const kv_ctx *ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

// ---------------------------------------------------------------------------
// Tracing
// ---------------------------------------------------------------------------

LaunchTimer::LaunchTimer(kv_ctx *c, const char *name) : ctx(c) {
    if (ctx == nullptr || !ctx->timing) return;
    cudaEvent_t ev[2];
    for (int i = 0; i < 2; ++i) {
        if (!ctx->event_pool.empty()) {
            ev[i] = ctx->event_pool.back();
            ctx->event_pool.pop_back();
        } else if (cudaEventCreate(&ev[i]) != cudaSuccess) {
            if (i == 1) ctx->event_pool.push_back(ev[0]);
            return;
        }
    }
    rec = kv_timing_rec{name, ev[0], ev[1]};
    cudaEventRecord(rec.start, ctx->stream);
}

LaunchTimer::~LaunchTimer() {
    if (rec.name == nullptr) return;
    cudaEventRecord(rec.stop, ctx->stream);
    ctx->timing_recs.push_back(rec);
}

extern "C" kv_status kv_ctx_set_timing(kv_ctx *ctx, int enable) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    ctx->timing = enable != 0;
    return KV_OK;
}

extern "C" kv_status kv_ctx_timing_read(kv_ctx *ctx, char *buf, size_t buflen) {
    if (ctx == nullptr || buf == nullptr || buflen == 0) return KV_ERR_INVALID_ARG;
    KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<std::string> names;
    std::vector<double> ms;
    std::vector<long> count;
    for (const kv_timing_rec &r : ctx->timing_recs) {
        float t = 0.f;
        cudaEventElapsedTime(&t, r.start, r.stop);
        size_t k = 0;
        while (k < names.size() && names[k] != r.name) ++k;
        if (k == names.size()) {
            names.emplace_back(r.name);
            ms.push_back(0.0);
            count.push_back(0);
        }
        ms[k] += t;
        count[k] += 1;
        ctx->event_pool.push_back(r.start);
        ctx->event_pool.push_back(r.stop);
    }
    ctx->timing_recs.clear();
    std::string out;
    char line[256];
    for (size_t k = 0; k < names.size(); ++k) {
        snprintf(line, sizeof line, "%s %ld %.6f\n", names[k].c_str(), count[k], ms[k]);
        out += line;
    }
    snprintf(buf, buflen, "%s", out.c_str());
    return KV_OK;
}

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------

extern "C" kv_status kv_plan_create(kv_ctx *ctx, const kv_geometry *g, kv_family family,
                                    kv_storage storage, kv_plan **out) {
    if (ctx == nullptr || g == nullptr || out == nullptr) return KV_ERR_INVALID_ARG;
    *out = nullptr;
    if (g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || g->nu <= 0 || g->nv <= 0 || g->n_views <= 0)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "sizes must be positive");
    if (g->src == nullptr || g->det_origin == nullptr)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "null source / detector array");
    KV_TRY(check_geometry_values(ctx, *g));
    if ((size_t)g->nx * g->ny >= (1ull << 31) || (size_t)g->nu * g->nv >= (1ull << 31))
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "slice or detector larger than 2^31 elements");
    if (family != KV_FAMILY_RC && family != KV_FAMILY_EXACT)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "bad family");
    if (storage != KV_STORAGE_F32 && storage != KV_STORAGE_BF16 && storage != KV_STORAGE_F16)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "bad storage");
    if (family == KV_FAMILY_RC && storage != KV_STORAGE_F32)
        return kv_fail(ctx, KV_ERR_UNSUPPORTED, "the reference-compatible family is FP32 only");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    kv_plan *plan = new (std::nothrow) kv_plan;
    if (plan == nullptr) return KV_ERR_OOM;
    plan->ctx = ctx;
    ctx->plans += 1;
    plan->g = *g;
    plan->src.assign(g->src, g->src + 3 * g->n_views);
    plan->det.assign(g->det_origin, g->det_origin + 3 * g->n_views);
    plan->g.src = plan->src.data();
    plan->g.det_origin = plan->det.data();
    plan->family = family;
    plan->storage = storage;
    plan->nvox = (size_t)g->nx * g->ny * g->nz;
    plan->nproj = (size_t)g->nu * g->nv * g->n_views;
    kv_status s = KV_OK;
    if (family == KV_FAMILY_EXACT) {
        s = exact_build_tables(plan, plan->src.data(), plan->det.data(), g->n_views, &plan->ex, &plan->hx);
        // the slab-staged forward projector where the geometry suits it: the
        // first shape of this list that fits (measured fastest first at the
        // chest-DT geometry; kv_plan_autotune can pick another)
        static const int shapes[][3] = {{8, 4, 2}, {4, 4, 3}, {4, 2, 3}, {2, 4, 3}, {2, 2, 2}};
        for (const auto &sh : shapes) {
            FwdSlabCfg c;
            if (s == KV_OK && fwd_slab_fit(plan, sh[0], sh[1], sh[2], fwd_slab_default_group(g->n_views), &c, nullptr)) {
                plan->fslab = c;
                break;
            }
        }
    } else {
        size_t bytes = 3 * sizeof(float) * g->n_views;
        if (cudaMalloc((void **)&plan->d_src, bytes) != cudaSuccess ||
            cudaMalloc((void **)&plan->d_org, bytes) != cudaSuccess) {
            s = kv_fail(ctx, KV_ERR_OOM, "plan tables");
        } else {
            cudaMemcpy(plan->d_src, plan->src.data(), bytes, cudaMemcpyHostToDevice);
            cudaMemcpy(plan->d_org, plan->det.data(), bytes, cudaMemcpyHostToDevice);
        }
    }
    if (s != KV_OK) {
        kv_plan_destroy(plan);
        return s;
    }
    *out = plan;
    return KV_OK;
}

extern "C" kv_status kv_plan_destroy(kv_plan *plan) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    cudaSetDevice(plan->ctx->device);
    cudaStreamSynchronize(plan->ctx->stream);
    exact_free_tables(&plan->ex);
    cudaFree(plan->d_src);
    cudaFree(plan->d_org);
    cudaFree(plan->d_vol);
    cudaFree(plan->d_proj);
    cudaFree(plan->d_ratio);
    cudaFree(plan->d_vol32);
    cudaFree(plan->d_proj32);
    cudaFree(plan->d_sens);
    cudaFree(plan->d_shift);
    if (plan->graph_exec) cudaGraphExecDestroy(plan->graph_exec);
    kv_ctx *ctx = plan->ctx;
    delete plan;
    kv_ctx_release_ref(ctx);
    return KV_OK;
}

void kv_ctx_release_ref(kv_ctx *ctx) {
    if (--ctx->plans == 0 && ctx->released) ctx_free(ctx);
}

extern "C" size_t kv_plan_volume_elems(const kv_plan *plan) { return plan ? plan->nvox : 0; }
extern "C" size_t kv_plan_proj_elems(const kv_plan *plan) { return plan ? plan->nproj : 0; }

// ---------------------------------------------------------------------------
// Operators
// ---------------------------------------------------------------------------

extern "C" kv_status kv_forward(kv_plan *plan, const float *volume, float *proj, kv_mem mem) {
    KV_TRY(check_common(plan, volume, proj, mem));
    float *vd, *pd;
    KV_TRY(stage_in(plan, volume, mem, &plan->d_vol32, plan->nvox, true, &vd));
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, false, &pd));
    if (mem == KV_MEM_HOST && plan->storage == KV_STORAGE_F32 && !stream_capturing(plan->ctx)) {
        // view chunks, each copied back while the next ones are projected
        KV_TRY(ensure_copy_stream(plan->ctx));
        auto fwd = [&](int v0, int n) -> kv_status {
            if (plan->family == KV_FAMILY_EXACT)
                return exact_forward_views_launch(plan, v0, n, FWD_PLAIN, FwdArgs{vd, nullptr, pd, nullptr, 1.f});
            const size_t off = (size_t)v0 * plan->g.nu * plan->g.nv;
            return rc_forward_launch(plan, plan->d_src + 3 * (size_t)v0, plan->d_org + 3 * (size_t)v0, n,
                                     RC_PLAIN, vd, nullptr, pd + off, 1.f);
        };
        return sync_both(plan->ctx, pieces_to_host_body(plan->ctx, plan->g.n_views,
                                                        (size_t)plan->g.nu * plan->g.nv, pd, proj, 1, fwd));
    }
    if (plan->family == KV_FAMILY_RC) {
        KV_TRY(rc_forward_launch(plan, plan->d_src, plan->d_org, plan->g.n_views, RC_PLAIN, vd, nullptr, pd, 1.f));
    } else if (plan->storage == KV_STORAGE_F32) {
        KV_TRY(exact_forward_launch(plan, plan->ex, plan->g.n_views, FWD_PLAIN, FwdArgs{vd, nullptr, pd, nullptr, 1.f}));
    } else {
        const size_t es = kv_storage_bytes(plan->storage);
        KV_TRY(ensure(plan->ctx, &plan->d_vol, plan->nvox * es));
        KV_TRY(ensure(plan->ctx, &plan->d_ratio, plan->nproj * es));
        KV_TRY(convert_launch(plan->ctx, vd, plan->d_vol, plan->nvox, plan->storage));
        KV_TRY(exact_forward_launch(plan, plan->ex, plan->g.n_views, FWD_PLAIN,
                                    FwdArgs{plan->d_vol, nullptr, plan->d_ratio, nullptr, 1.f}));
        KV_TRY(convert_back_launch(plan->ctx, plan->d_ratio, pd, plan->nproj, plan->storage));
    }
    return stage_out(plan, proj, mem, pd, plan->nproj);
}

extern "C" kv_status kv_forward_single(kv_plan *plan, const float *volume, const float src[3],
                                       const float det_origin[3], float *proj, kv_mem mem) {
    KV_TRY(check_common(plan, volume, proj, mem));
    if (src == nullptr || det_origin == nullptr) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "null position");
    const size_t nout = (size_t)plan->g.nu * plan->g.nv;
    float *vd, *pd;
    KV_TRY(stage_in(plan, volume, mem, &plan->d_vol32, plan->nvox, true, &vd));
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, false, &pd));
    if (plan->family == KV_FAMILY_RC) {
        float *d6 = nullptr;
        KV_CHECK_CUDA(plan->ctx, cudaMallocAsync((void **)&d6, 6 * sizeof(float), plan->ctx->stream));
        float h6[6] = {src[0], src[1], src[2], det_origin[0], det_origin[1], det_origin[2]};
        KV_CHECK_CUDA(plan->ctx, cudaMemcpyAsync(d6, h6, sizeof h6, cudaMemcpyHostToDevice, plan->ctx->stream));
        kv_status s = rc_forward_launch(plan, d6, d6 + 3, 1, RC_PLAIN, vd, nullptr, pd, 1.f);
        cudaFreeAsync(d6, plan->ctx->stream);
        KV_TRY(s);
    } else {
        if (plan->storage != KV_STORAGE_F32) return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "single-view forward is FP32 only");
        ExactTables t;
        KV_TRY(exact_build_tables(plan, src, det_origin, 1, &t, nullptr));
        // the plan's slab boxes are sized for its own views: this view takes
        // the one-thread-per-ray kernel
        const FwdSlabCfg keep = plan->fslab;
        plan->fslab.R = 0;
        kv_status s = exact_forward_launch(plan, t, 1, FWD_PLAIN, FwdArgs{vd, nullptr, pd, nullptr, 1.f});
        plan->fslab = keep;
        cudaStreamSynchronize(plan->ctx->stream);
        exact_free_tables(&t);
        KV_TRY(s);
    }
    return stage_out(plan, proj, mem, pd, nout);
}

extern "C" kv_status kv_back(kv_plan *plan, const float *proj, float *volume, kv_mem mem) {
    KV_TRY(check_common(plan, proj, volume, mem));
    float *pd, *vd;
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, true, &pd));
    KV_TRY(stage_in(plan, volume, mem, &plan->d_vol32, plan->nvox, false, &vd));
    if (mem == KV_MEM_HOST && plan->storage == KV_STORAGE_F32 && !stream_capturing(plan->ctx)) {
        // slabs of slices, each copied back while the next ones are computed
        KV_TRY(ensure_copy_stream(plan->ctx));
        if (plan->family == KV_FAMILY_EXACT) {
            KV_TRY(ensure(plan->ctx, &plan->d_ratio, plan->nproj * sizeof(float)));
            KV_TRY(exact_prescale_launch(plan, pd, plan->d_ratio));
        }
        auto back = [&](int z0, int n) -> kv_status {
            if (plan->family == KV_FAMILY_EXACT)
                return exact_back_slab_launch(plan, BACK_PLAIN, BackArgs{plan->d_ratio, vd, nullptr, 1.f}, z0, n);
            return rc_back_slab_launch(plan, RC_PLAIN, pd, vd, z0, n);
        };
        return sync_both(plan->ctx, pieces_to_host_body(plan->ctx, plan->g.nz, (size_t)plan->g.nx * plan->g.ny,
                                                        vd, volume, 1, back));
    }
    if (plan->family == KV_FAMILY_RC) {
        KV_TRY(rc_back_launch(plan, RC_PLAIN, pd, vd));
    } else {
        const size_t es = kv_storage_bytes(plan->storage);
        KV_TRY(ensure(plan->ctx, &plan->d_ratio, plan->nproj * es));
        KV_TRY(exact_prescale_launch(plan, pd, plan->d_ratio));
        if (plan->storage == KV_STORAGE_F32) {
            KV_TRY(exact_back_launch(plan, BACK_PLAIN, BackArgs{plan->d_ratio, vd, nullptr, 1.f}));
        } else {
            KV_TRY(ensure(plan->ctx, &plan->d_vol, plan->nvox * es));
            KV_TRY(exact_back_launch(plan, BACK_PLAIN, BackArgs{plan->d_ratio, plan->d_vol, nullptr, 1.f}));
            KV_TRY(convert_back_launch(plan->ctx, plan->d_vol, vd, plan->nvox, plan->storage));
        }
    }
    return stage_out(plan, volume, mem, vd, plan->nvox);
}

extern "C" kv_status kv_fbp(kv_plan *plan, const float *proj, float *volume, int32_t half_taps, kv_mem mem) {
    KV_TRY(check_common(plan, proj, volume, mem));
    if (plan->family != KV_FAMILY_EXACT || plan->storage != KV_STORAGE_F32)
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "filtered backprojection needs the EXACT family, FP32 storage");
    if (half_taps < 1 || half_taps > KV_FBP_MAX_HALF_TAPS)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "half_taps must be 1..%d (got %d)", KV_FBP_MAX_HALF_TAPS,
                       half_taps);
    float *pd, *vd;
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, true, &pd));
    KV_TRY(stage_in(plan, volume, mem, &plan->d_vol32, plan->nvox, false, &vd));
    KV_TRY(ensure_sens(plan));
    KV_TRY(ensure(plan->ctx, &plan->d_ratio, plan->nproj * sizeof(float)));
    float *filtered = nullptr;
    KV_CHECK_CUDA(plan->ctx, cudaMallocAsync((void **)&filtered, plan->nproj * sizeof(float), plan->ctx->stream));
    kv_status st = ramp_filter_launch(plan, pd, filtered, half_taps);
    if (st == KV_OK) st = exact_prescale_launch(plan, filtered, plan->d_ratio);
    cudaFreeAsync(filtered, plan->ctx->stream);
    KV_TRY(st);
    // volume = 0 + 1 * A^T(y) / A^T 1: the SART-mode update epilogue from zero
    KV_TRY(fill_launch(plan->ctx, vd, plan->nvox, 0.f));
    KV_TRY(exact_back_launch(plan, BACK_SART, BackArgs{plan->d_ratio, vd, plan->d_sens, 1.f}));
    return stage_out(plan, volume, mem, vd, plan->nvox);
}

extern "C" kv_status kv_sensitivity(kv_plan *plan, double *sens, kv_mem mem) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (sens == nullptr) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "null buffer");
    if (plan->family != KV_FAMILY_EXACT)
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "the sensitivity image is defined for the EXACT family");
    KV_CHECK_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
    KV_TRY(ensure_sens(plan));
    KV_CHECK_CUDA(plan->ctx, cudaMemcpyAsync(sens, plan->d_sens, plan->nvox * sizeof(double),
                                             mem == KV_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                                             plan->ctx->stream));
    if (mem == KV_MEM_HOST) KV_CHECK_CUDA(plan->ctx, cudaStreamSynchronize(plan->ctx->stream));
    return KV_OK;
}

extern "C" kv_status kv_shift_and_add(kv_plan *plan, const float *proj, float *slices, kv_mem mem) {
    KV_TRY(check_common(plan, proj, slices, mem));
    std::vector<int32_t> sh((size_t)plan->g.nz * plan->g.n_views);
    KV_TRY(saa_shifts(plan->ctx, plan->g, plan->family, sh.data()));
    // a shift of nv rows or more moves every row off the detector (zero
    // padding): +-nv gives the same sum and keeps the kernel's row index
    // v + shift far from overflow
    for (int32_t &s : sh) s = std::min(std::max(s, -plan->g.nv), plan->g.nv);
    const size_t nout = (size_t)plan->g.nz * plan->g.nv * plan->g.nu;
    KV_TRY(ensure(plan->ctx, &plan->d_shift, sh.size() * sizeof(int32_t)));
    KV_CHECK_CUDA(plan->ctx, cudaMemcpyAsync(plan->d_shift, sh.data(), sh.size() * sizeof(int32_t),
                                             cudaMemcpyHostToDevice, plan->ctx->stream));
    float *pd, *od = nullptr;
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, true, &pd));
    if (mem == KV_MEM_DEVICE) od = slices;
    else KV_CHECK_CUDA(plan->ctx, cudaMallocAsync((void **)&od, nout * sizeof(float), plan->ctx->stream));
    kv_status s = saa_launch(plan, plan->d_shift, sh.data(), pd, od);
    if (s == KV_OK && mem == KV_MEM_HOST) s = stage_out(plan, slices, mem, od, nout);
    if (mem == KV_MEM_HOST) cudaFreeAsync(od, plan->ctx->stream);
    return s;
}

extern "C" kv_status kv_shift_and_add_shifts(const kv_geometry *geom, kv_family family, int32_t *shifts) {
    if (geom == nullptr || shifts == nullptr || geom->src == nullptr || geom->det_origin == nullptr)
        return KV_ERR_INVALID_ARG;
    if (family != KV_FAMILY_RC && family != KV_FAMILY_EXACT) return KV_ERR_INVALID_ARG;
    return saa_shifts(nullptr, *geom, family, shifts);
}

extern "C" kv_status kv_phantom_ellipsoids(kv_ctx *ctx, int32_t nx, int32_t ny, int32_t nz, float dx,
                                           float dy, float dz, const float *params, int32_t n,
                                           float *volume, kv_mem mem) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (params == nullptr || volume == nullptr || n < 0 || nx <= 0 || ny <= 0 || nz <= 0)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "bad phantom arguments");
    if (mem != KV_MEM_HOST && mem != KV_MEM_DEVICE) return kv_fail(ctx, KV_ERR_INVALID_ARG, "bad kv_mem");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t nvox = (size_t)nx * ny * nz;
    float *dp = nullptr, *dv = nullptr;
    KV_CHECK_CUDA(ctx, cudaMallocAsync((void **)&dp, (size_t)16 * (n > 0 ? n : 1) * sizeof(float), ctx->stream));
    if (n > 0) {
        cudaMemcpyKind kind = mem == KV_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        KV_CHECK_CUDA(ctx, cudaMemcpyAsync(dp, params, (size_t)16 * n * sizeof(float), kind, ctx->stream));
    }
    if (mem == KV_MEM_DEVICE) dv = volume;
    else KV_CHECK_CUDA(ctx, cudaMallocAsync((void **)&dv, nvox * sizeof(float), ctx->stream));
    kv_status s = phantom_launch(ctx, nx, ny, nz, dx, dy, dz, dp, n, dv);
    if (s == KV_OK && mem == KV_MEM_HOST) {
        cudaError_t e = cudaMemcpyAsync(volume, dv, nvox * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) s = kv_fail(ctx, KV_ERR_CUDA, "phantom copy-out: %s", cudaGetErrorString(e));
    }
    cudaFreeAsync(dp, ctx->stream);
    if (mem == KV_MEM_HOST) cudaFreeAsync(dv, ctx->stream);
    return s;
}

extern "C" kv_status kv_uniform_volume(kv_plan *plan, float *volume, kv_mem mem) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (volume == nullptr) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "null buffer");
    if (mem == KV_MEM_HOST) {
        for (size_t i = 0; i < plan->nvox; ++i) volume[i] = 1.f;
        return KV_OK;
    }
    KV_CHECK_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
    return fill_launch(plan->ctx, volume, plan->nvox, 1.f);
}

// ---------------------------------------------------------------------------
// Iterative drivers
// ---------------------------------------------------------------------------

kv_status rc_residual_launch(kv_plan *plan, const float *q, const float *p, double *red);
kv_status rc_ratio_launch(kv_plan *plan, int mode, const float *p, float *q, float relax);

namespace {

// MLEM (mlem = true) or SART/ART (mlem = false) on device buffers: p, x are
// float32 (RC or F32 storage) or storage-typed (EXACT mixed precision).
kv_status iterate(kv_plan *plan, const void *p, void *x, int iters, float relax, bool mlem,
                  kv_iter_cb cb, void *user);

// Without a callback (and without tracing) the iteration loop is captured once
// as a CUDA graph on the context's own stream and launched on the call's
// stream; the executable graph is kept and relaunched while the buffers and
// parameters stay the same.
long long slab_key(const FwdSlabCfg &c) {
    return (((long long)c.R * 16 + c.S) * 8 + c.stages) * 65536 + c.group;
}

kv_status iterate_graph(kv_plan *plan, const void *p, void *x, int iters, float relax, bool mlem) {
    kv_ctx *ctx = plan->ctx;
    const bool same = plan->graph_exec != nullptr && plan->graph_p == p && plan->graph_x == x &&
                      plan->graph_iters == iters && plan->graph_mlem == (int)mlem && plan->graph_relax == relax &&
                      plan->graph_fb == plan->fwd_by && plan->graph_bb == plan->back_by &&
                      plan->graph_slab == slab_key(plan->fslab) && plan->graph_br == plan->back_rows &&
                      plan->graph_bs == plan->back_slices &&
                      plan->graph_bst == plan->bstage.R * 16 + plan->bstage.stages;
    if (!same) {
        if (plan->graph_exec != nullptr) {
            KV_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaGraphExecDestroy(plan->graph_exec);
            plan->graph_exec = nullptr;
        }
        cudaStream_t user_stream = ctx->stream;
        ctx->stream = ctx->own_stream;
        KV_CHECK_CUDA(ctx, cudaStreamBeginCapture(ctx->own_stream, cudaStreamCaptureModeThreadLocal));
        kv_status s = iterate(plan, p, x, iters, relax, mlem, nullptr, nullptr);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->own_stream, &graph);
        ctx->stream = user_stream;
        if (s != KV_OK) {
            if (graph) cudaGraphDestroy(graph);
            return s;
        }
        if (e != cudaSuccess) return kv_fail(ctx, KV_ERR_CUDA, "iteration capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&plan->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            plan->graph_exec = nullptr;
            return kv_fail(ctx, KV_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        }
        plan->graph_p = p;
        plan->graph_x = x;
        plan->graph_iters = iters;
        plan->graph_mlem = (int)mlem;
        plan->graph_relax = relax;
        plan->graph_fb = plan->fwd_by;
        plan->graph_bb = plan->back_by;
        plan->graph_slab = slab_key(plan->fslab);
        plan->graph_br = plan->back_rows;
        plan->graph_bs = plan->back_slices;
        plan->graph_bst = plan->bstage.R * 16 + plan->bstage.stages;
    }
    KV_CHECK_CUDA(ctx, cudaGraphLaunch(plan->graph_exec, ctx->stream));
    return KV_OK;
}

kv_status iterate(kv_plan *plan, const void *p, void *x, int iters, float relax, bool mlem,
                  kv_iter_cb cb, void *user) {
    kv_ctx *ctx = plan->ctx;
    const size_t es = kv_storage_bytes(plan->storage);
    KV_TRY(ensure(ctx, &plan->d_ratio, plan->nproj * es));
    if (plan->family == KV_FAMILY_EXACT) KV_TRY(ensure_sens(plan));
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(ctx->stream, &cs);
    if (cb == nullptr && !ctx->timing && iters >= 2 && cs == cudaStreamCaptureStatusNone)
        return iterate_graph(plan, p, x, iters, relax, mlem);
    for (int it = 0; it < iters; ++it) {
        if (plan->family == KV_FAMILY_EXACT) {
            FwdArgs fa{x, p, plan->d_ratio, cb ? ctx->d_red : nullptr, relax};
            KV_TRY(exact_forward_launch(plan, plan->ex, plan->g.n_views, mlem ? FWD_MLEM : FWD_SART, fa));
        } else if (cb) {
            KV_TRY(rc_forward_launch(plan, plan->d_src, plan->d_org, plan->g.n_views, RC_PLAIN, (const float *)x,
                                     nullptr, (float *)plan->d_ratio, relax));
            KV_TRY(rc_residual_launch(plan, (const float *)plan->d_ratio, (const float *)p, ctx->d_red));
        } else {
            KV_TRY(rc_forward_launch(plan, plan->d_src, plan->d_org, plan->g.n_views, mlem ? RC_MLEM : RC_ART,
                                     (const float *)x, (const float *)p, (float *)plan->d_ratio, relax));
        }
        if (cb) {
            double res = 0.0, ll = 0.0;
            KV_TRY(residual_from_red(ctx, &res, &ll));
            if (cb(it, res, ll, user) != 0) return KV_OK;
            if (plan->family == KV_FAMILY_RC)
                KV_TRY(rc_ratio_launch(plan, mlem ? RC_MLEM : RC_ART, (const float *)p, (float *)plan->d_ratio, relax));
        }
        if (plan->family == KV_FAMILY_EXACT) {
            BackArgs ba{plan->d_ratio, x, plan->d_sens, relax};
            KV_TRY(exact_back_launch(plan, mlem ? BACK_MLEM : BACK_SART, ba));
        } else {
            KV_TRY(rc_back_launch(plan, mlem ? RC_MLEM : RC_ART, (const float *)plan->d_ratio, (float *)x));
        }
    }
    return KV_OK;
}

// Host-buffer MLEM / SART (both families, FP32 storage) without a callback.
// The volume and then the projections, in growing view chunks, go up on the
// context's copy stream; the first forward projection runs chunk by chunk,
// each chunk as soon as its projections have landed.  The last
// backprojection runs in shrinking slabs of slices and each slab is copied
// back while the next ones are computed.  Per ray and per voxel the
// arithmetic is that of the whole-volume launches, so the result equals the
// device-buffer call bit for bit.

// The fused update step of either family on views [v0, v0 + n) (forward +
// ratio) and on slices [z0, z0 + n) (backprojection + update).
kv_status update_forward_views(kv_plan *plan, bool mlem, const float *pd, const float *xd, float relax, int v0,
                               int n) {
    if (plan->family == KV_FAMILY_EXACT)
        return exact_forward_views_launch(plan, v0, n, mlem ? FWD_MLEM : FWD_SART,
                                          FwdArgs{xd, pd, plan->d_ratio, nullptr, relax});
    const size_t off = (size_t)v0 * plan->g.nu * plan->g.nv;
    return rc_forward_launch(plan, plan->d_src + 3 * (size_t)v0, plan->d_org + 3 * (size_t)v0, n,
                             mlem ? RC_MLEM : RC_ART, xd, pd + off, (float *)plan->d_ratio + off, relax);
}

kv_status update_back_slab(kv_plan *plan, bool mlem, float *xd, float relax, int z0, int n) {
    if (plan->family == KV_FAMILY_EXACT)
        return exact_back_slab_launch(plan, mlem ? BACK_MLEM : BACK_SART,
                                      BackArgs{plan->d_ratio, xd, plan->d_sens, relax}, z0, n);
    return rc_back_slab_launch(plan, mlem ? RC_MLEM : RC_ART, (const float *)plan->d_ratio, xd, z0, n);
}

kv_status overlapped_body(kv_plan *plan, const float *proj, float *volume, int iters, float relax, bool mlem) {
    kv_ctx *ctx = plan->ctx;
    const kv_geometry &g = plan->g;
    const size_t D = (size_t)g.nu * g.nv, plane = (size_t)g.nx * g.ny;
    float *pd = plan->d_proj32, *xd = plan->d_vol32;
    cudaStream_t cs = ctx->copy_stream, st = ctx->stream;
    cudaEvent_t *ev = ctx->copy_events.data();
    // earlier work on the context stream may still read the staging buffers
    KV_CHECK_CUDA(ctx, cudaEventRecord(ev[0], st));
    KV_CHECK_CUDA(ctx, cudaStreamWaitEvent(cs, ev[0], 0));
    KV_CHECK_CUDA(ctx, cudaMemcpyAsync(xd, volume, plan->nvox * sizeof(float), cudaMemcpyHostToDevice, cs));
    const std::vector<int> vb = overlap_bounds(g.n_views, false);
    for (int c = 0; c + 1 < (int)vb.size(); ++c) {
        const int v0 = vb[c], n = vb[c + 1] - vb[c];
        KV_CHECK_CUDA(ctx, cudaMemcpyAsync(pd + v0 * D, proj + v0 * D, n * D * sizeof(float),
                                           cudaMemcpyHostToDevice, cs));
        KV_CHECK_CUDA(ctx, cudaEventRecord(ev[1 + c], cs));
        KV_CHECK_CUDA(ctx, cudaStreamWaitEvent(st, ev[1 + c], 0));
        KV_TRY(update_forward_views(plan, mlem, pd, xd, relax, v0, n));
    }
    if (iters > 1) {
        KV_TRY(update_back_slab(plan, mlem, xd, relax, 0, g.nz));
        if (iters > 2) KV_TRY(iterate(plan, pd, xd, iters - 2, relax, mlem, nullptr, nullptr));
        KV_TRY(update_forward_views(plan, mlem, pd, xd, relax, 0, g.n_views));
    }
    auto back = [&](int z0, int n) { return update_back_slab(plan, mlem, xd, relax, z0, n); };
    return pieces_to_host_body(ctx, g.nz, plane, xd, volume, 1 + kOverlapChunks, back);
}

kv_status driver_overlapped(kv_plan *plan, const float *proj, float *volume, int iters, float relax, bool mlem) {
    kv_ctx *ctx = plan->ctx;
    KV_TRY(ensure(ctx, &plan->d_proj32, plan->nproj * sizeof(float)));
    KV_TRY(ensure(ctx, &plan->d_vol32, plan->nvox * sizeof(float)));
    KV_TRY(ensure(ctx, &plan->d_ratio, plan->nproj * sizeof(float)));
    if (plan->family == KV_FAMILY_EXACT) KV_TRY(ensure_sens(plan));
    KV_TRY(ensure_copy_stream(ctx));
    return sync_both(ctx, overlapped_body(plan, proj, volume, iters, relax, mlem));
}

kv_status driver(kv_plan *plan, const float *proj, float *volume, int iters, float relax, kv_mem mem,
                 kv_iter_cb cb, void *user, bool mlem) {
    KV_TRY(check_common(plan, proj, volume, mem));
    if (iters < 0) return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "negative iteration count");
    if (!std::isfinite(relax)) return kv_fail(plan->ctx, KV_ERR_NUMERIC, "non-finite relaxation");
    if (mem == KV_MEM_HOST && plan->storage == KV_STORAGE_F32 && cb == nullptr && iters >= 1 &&
        !stream_capturing(plan->ctx))
        return driver_overlapped(plan, proj, volume, iters, relax, mlem);
    float *pd, *xd;
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, true, &pd));
    KV_TRY(stage_in(plan, volume, mem, &plan->d_vol32, plan->nvox, true, &xd));
    if (plan->storage == KV_STORAGE_F32) {
        KV_TRY(iterate(plan, pd, xd, iters, relax, mlem, cb, user));
    } else {
        const size_t es = kv_storage_bytes(plan->storage);
        KV_TRY(ensure(plan->ctx, &plan->d_vol, plan->nvox * es));
        KV_TRY(ensure(plan->ctx, &plan->d_proj, plan->nproj * es));
        KV_TRY(convert_launch(plan->ctx, pd, plan->d_proj, plan->nproj, plan->storage));
        KV_TRY(convert_launch(plan->ctx, xd, plan->d_vol, plan->nvox, plan->storage));
        KV_TRY(iterate(plan, plan->d_proj, plan->d_vol, iters, relax, mlem, cb, user));
        KV_TRY(convert_back_launch(plan->ctx, plan->d_vol, xd, plan->nvox, plan->storage));
    }
    return stage_out(plan, volume, mem, xd, plan->nvox);
}

}  // namespace

extern "C" kv_status kv_mlem(kv_plan *plan, const float *proj, float *volume, int iters, float relax,
                             kv_mem mem, kv_iter_cb cb, void *user) {
    return driver(plan, proj, volume, iters, relax, mem, cb, user, true);
}

extern "C" kv_status kv_sart(kv_plan *plan, const float *proj, float *volume, int iters, float relax,
                             kv_mem mem, kv_iter_cb cb, void *user) {
    return driver(plan, proj, volume, iters, relax, mem, cb, user, false);
}

extern "C" kv_status kv_residual(kv_plan *plan, const float *proj, const float *volume, kv_mem mem,
                                 double *rel_residual, double *loglik) {
    KV_TRY(check_common(plan, proj, volume, mem));
    float *pd, *xd;
    KV_TRY(stage_in(plan, proj, mem, &plan->d_proj32, plan->nproj, true, &pd));
    KV_TRY(stage_in(plan, volume, mem, &plan->d_vol32, plan->nvox, true, &xd));
    if (plan->family == KV_FAMILY_EXACT) {
        const void *pv = pd, *xv = xd;
        if (plan->storage != KV_STORAGE_F32) {
            const size_t es = kv_storage_bytes(plan->storage);
            KV_TRY(ensure(plan->ctx, &plan->d_vol, plan->nvox * es));
            KV_TRY(ensure(plan->ctx, &plan->d_proj, plan->nproj * es));
            KV_TRY(convert_launch(plan->ctx, pd, plan->d_proj, plan->nproj, plan->storage));
            KV_TRY(convert_launch(plan->ctx, xd, plan->d_vol, plan->nvox, plan->storage));
            pv = plan->d_proj;
            xv = plan->d_vol;
        }
        FwdArgs fa{xv, pv, nullptr, plan->ctx->d_red, 1.f};
        KV_TRY(exact_forward_launch(plan, plan->ex, plan->g.n_views, FWD_RESID, fa));
    } else {
        KV_TRY(ensure(plan->ctx, &plan->d_ratio, plan->nproj * sizeof(float)));
        KV_TRY(rc_forward_launch(plan, plan->d_src, plan->d_org, plan->g.n_views, RC_PLAIN, xd, nullptr,
                                 (float *)plan->d_ratio, 1.f));
        KV_TRY(rc_residual_launch(plan, (const float *)plan->d_ratio, pd, plan->ctx->d_red));
    }
    return residual_from_red(plan->ctx, rel_residual, loglik);
}

// ---------------------------------------------------------------------------
// Batched solves and tuning
// ---------------------------------------------------------------------------

extern "C" kv_status kv_batch_mlem(kv_ctx *ctx, int n, kv_plan *const *plans, const float *const *projections,
                                   float *const *volumes, int iterations, float relax, kv_mem mem) {
    if (ctx == nullptr) return KV_ERR_INVALID_ARG;
    if (n <= 0 || plans == nullptr || projections == nullptr || volumes == nullptr)
        return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_batch_mlem: empty batch or null arrays");
    if (iterations < 0) return kv_fail(ctx, KV_ERR_INVALID_ARG, "negative iteration count");
    if (!std::isfinite(relax)) return kv_fail(ctx, KV_ERR_NUMERIC, "non-finite relaxation");
    if (mem != KV_MEM_HOST && mem != KV_MEM_DEVICE) return kv_fail(ctx, KV_ERR_INVALID_ARG, "bad kv_mem");
    KV_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    for (int i = 0; i < n; ++i) {
        kv_plan *pl = plans[i];
        if (pl == nullptr || projections[i] == nullptr || volumes[i] == nullptr)
            return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_batch_mlem: null plan or buffer %d", i);
        if (pl->ctx != ctx) return kv_fail(ctx, KV_ERR_INVALID_ARG, "kv_batch_mlem: plan %d has another context", i);
        if (pl->family != KV_FAMILY_EXACT || pl->storage != KV_STORAGE_F32)
            return kv_fail(ctx, KV_ERR_UNSUPPORTED, "kv_batch_mlem: EXACT / FP32 plans only (plan %d)", i);
    }
    const int by = plans[0]->fwd_by, bb = plans[0]->back_by;
    std::vector<const float *> pd(n);
    std::vector<float *> xd(n);
    for (int i = 0; i < n; ++i) {
        kv_plan *pl = plans[i];
        KV_TRY(ensure(ctx, &pl->d_ratio, pl->nproj * sizeof(float)));
        KV_TRY(ensure_sens(pl));
        float *a, *b;
        KV_TRY(stage_in(pl, projections[i], mem, &pl->d_proj32, pl->nproj, true, &a));
        KV_TRY(stage_in(pl, volumes[i], mem, &pl->d_vol32, pl->nvox, true, &b));
        pd[i] = a;
        xd[i] = b;
    }
    if (iterations > 0) KV_TRY(exact_batch_mlem_launch(ctx, n, plans, pd.data(), xd.data(), iterations, relax, by, bb));
    for (int i = 0; i < n; ++i) KV_TRY(stage_out(plans[i], volumes[i], mem, xd[i], plans[i]->nvox));
    return KV_OK;
}

extern "C" kv_status kv_plan_autotune(kv_plan *plan) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (plan->family != KV_FAMILY_EXACT)
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "the autotuner covers the EXACT kernels");
    KV_CHECK_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
    return exact_autotune(plan);
}

extern "C" kv_status kv_plan_get_tuning(const kv_plan *plan, int *fwd_rows, int *back_rows) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (fwd_rows) *fwd_rows = plan->fwd_by;
    if (back_rows) *back_rows = plan->back_by;
    return KV_OK;
}

extern "C" kv_status kv_plan_set_tuning(kv_plan *plan, int fwd_rows, int back_rows) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (fwd_rows < 1 || fwd_rows > 8 || back_rows < 1 || back_rows > 8)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG, "tuning out of range (1..8 rows of 32 threads)");
    plan->fwd_by = fwd_rows;
    plan->back_by = back_rows;
    return KV_OK;
}

extern "C" kv_status kv_plan_get_slab(const kv_plan *plan, int *rays_per_thread, int *slices, int *stages,
                                      int *view_group) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (rays_per_thread) *rays_per_thread = plan->fslab.R;
    if (slices) *slices = plan->fslab.S;
    if (stages) *stages = plan->fslab.stages;
    if (view_group) *view_group = plan->fslab.group;
    return KV_OK;
}

extern "C" kv_status kv_plan_set_slab(kv_plan *plan, int rays_per_thread, int slices, int stages, int view_group) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (plan->family != KV_FAMILY_EXACT)
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "the slab forward projector is an EXACT-family kernel");
    if (rays_per_thread == 0) {
        plan->fslab = FwdSlabCfg{};
        return KV_OK;
    }
    FwdSlabCfg c;
    std::string why;
    if (!fwd_slab_fit(plan, rays_per_thread, slices, stages, view_group, &c, &why))
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "slab shape (%d, %d, %d, %d) does not fit: %s",
                       rays_per_thread, slices, stages, view_group, why.c_str());
    plan->fslab = c;
    return KV_OK;
}

extern "C" kv_status kv_plan_get_back_staging(const kv_plan *plan, int *rows_per_thread, int *stages,
                                              int *patch_cols, int *patch_rows) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (rows_per_thread) *rows_per_thread = plan->bstage.R;
    if (stages) *stages = plan->bstage.stages;
    if (patch_cols) *patch_cols = plan->bstage.BU;
    if (patch_rows) *patch_rows = plan->bstage.BV;
    return KV_OK;
}

extern "C" kv_status kv_plan_set_back_staging(kv_plan *plan, int rows_per_thread, int stages) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (rows_per_thread == 0) {
        plan->bstage = BackStageCfg{};
        return KV_OK;
    }
    if (plan->family != KV_FAMILY_EXACT)
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "the staged backprojector is an EXACT-family kernel");
    BackStageCfg c;
    std::string why;
    if (!back_stage_fit(plan, rows_per_thread, stages, &c, &why))
        return kv_fail(plan->ctx, KV_ERR_UNSUPPORTED, "%s", why.c_str());
    plan->bstage = c;
    return KV_OK;
}

extern "C" kv_status kv_plan_get_back_shape(const kv_plan *plan, int *rows_per_thread, int *slices_per_thread) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    if (rows_per_thread) *rows_per_thread = plan->back_rows;
    if (slices_per_thread) *slices_per_thread = plan->back_slices;
    return KV_OK;
}

extern "C" kv_status kv_plan_set_back_shape(kv_plan *plan, int rows_per_thread, int slices_per_thread) {
    if (plan == nullptr) return KV_ERR_INVALID_ARG;
    const bool ok = rows_per_thread == 0 || (rows_per_thread == 1 && slices_per_thread == 1) ||
                    ((rows_per_thread == 2 || rows_per_thread == 4) &&
                     (slices_per_thread == 1 || slices_per_thread == 2)) ||
                    (rows_per_thread == 8 && slices_per_thread == 1);
    if (!ok)
        return kv_fail(plan->ctx, KV_ERR_INVALID_ARG,
                       "gather backprojector shape must be rows 0, (1, 1), (2, 1), (2, 2), (4, 1), (4, 2) or (8, 1)");
    if (rows_per_thread == 0) slices_per_thread = 1;
    plan->back_rows = rows_per_thread;
    plan->back_slices = slices_per_thread;
    return KV_OK;
}
