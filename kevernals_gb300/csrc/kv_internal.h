// kv_internal.h -- shared definitions of the kvtomo CUDA engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdarg>
#include <cstdint>
#include <string>
#include <vector>

#include "kvtomo.h"

// ---------------------------------------------------------------------------
// Context and plan
// ---------------------------------------------------------------------------

struct kv_timing_rec {
    const char *name;
    cudaEvent_t start, stop;
};

struct kv_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;   // stream in use
    cudaStream_t own_stream = nullptr;
    std::string last_error;
    double *d_red = nullptr;         // 8 doubles for FP64 reductions
    int *d_status = nullptr;         // error bits set by kernels that check themselves (0: fine)
    // lifetime: plans hold a reference; kv_ctx_destroy only releases the
    // caller's, the context is freed with its last plan
    int plans = 0;
    bool released = false;
    // per-kernel tracing (kv_ctx_set_timing)
    bool timing = false;
    std::vector<kv_timing_rec> timing_recs;
    std::vector<cudaEvent_t> event_pool;
    // host-buffer MLEM / SART: copies overlapped with the first forward and
    // the last backprojection (created on first use)
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> copy_events;
};

// Brackets one kernel launch with CUDA events on the context stream when the
// context's tracing is enabled; a no-op otherwise.
struct LaunchTimer {
    kv_ctx *ctx;
    kv_timing_rec rec{nullptr, nullptr, nullptr};
    LaunchTimer(kv_ctx *c, const char *name);
    ~LaunchTimer();
};

// Per-view geometry tables of the EXACT family, computed on the host in
// double and stored as float (see kv_plan.cu).
//   xt[p][u] = {fxb, gx, ixx, ax}, xi[p][u] = ib : the x coordinate of ray
//              column u at relative height hr is ib + fmaf(gx, hr, fxb) voxels;
//              ixx = -1/(gx*dh) converts a plane offset into the slice-local
//              parameter t; ax = src.x - pixel.x (mm).
//   yt, yi     the same for detector rows v.
//   hr[p][k]   height of z-plane k relative to the volume centre, divided by
//              the source-detector distance H (k = 0..nz).
//   vinfo[p]   {H*H, dh = dz/H, 0, 0}.
//   rng[p][k]  {Ax, 1/Bx, Ay, 1/By}: at plane k the x coordinate of column u
//              is Ax + Bx*u (same for y); used to bound the candidate rays of a
//              voxel in the gather backprojector.
struct ExactTables {
    float4 *xt = nullptr;
    int *xi = nullptr;
    float4 *yt = nullptr;
    int *yi = nullptr;
    float *hr = nullptr;
    float4 *vinfo = nullptr;
    float4 *rng = nullptr;
};

// Host copies of the same tables (the slab forward projector sizes its
// shared-memory boxes from them with the kernel's own float arithmetic).
struct ExactHostTables {
    std::vector<float4> xt, yt, rng;
    std::vector<int> xi, yi;
    std::vector<float> hr;
};

// Launch shape of the slab-staged EXACT forward projector (kv_fwd_slab.cu);
// R == 0: the plan uses the one-thread-per-ray kernel instead.
struct FwdSlabCfg {
    int R = 0;          // rays per thread along v: a CTA covers 32 x 8R rays
    int S = 0;          // slices per slab
    int stages = 0;     // slab boxes in flight
    int group = 0;      // consecutive views launched together (L2 reuse)
    int BX = 0, BY = 0; // box extent in voxels
    size_t smem = 0;    // dynamic shared memory per CTA
};

// Shape of the TMA-staged EXACT backprojector (kv_back_stage.cu, FP32
// storage); R == 0: the plan uses exact_back_r_kernel / exact_back_kernel.
struct BackStageCfg {
    int R = 0;          // voxel rows per thread: a CTA covers 32 x 8R voxels of one slice
    int stages = 0;     // detector patches in flight
    int BU = 0, BV = 0; // patch extent in detector columns / rows
    size_t smem = 0;    // dynamic shared memory per CTA
};

struct kv_plan {
    kv_ctx *ctx = nullptr;
    kv_geometry g{};
    std::vector<float> src, det;     // host copies of the per-view arrays
    kv_family family = KV_FAMILY_EXACT;
    kv_storage storage = KV_STORAGE_F32;
    size_t nvox = 0, nproj = 0;

    // device geometry
    ExactTables ex;                  // EXACT family
    ExactHostTables hx;              // host copies of ex
    FwdSlabCfg fslab;                // slab forward projector (R == 0: not used)
    BackStageCfg bstage;             // staged backprojector (R == 0: not used)
    float *d_src = nullptr;          // RC family: [P][3] sources (float3 layout)
    float *d_org = nullptr;          // RC family: [P][3] detector origins

    // workspace (allocated on demand, kept for the plan's lifetime)
    void *d_vol = nullptr;           // volume in storage type
    void *d_proj = nullptr;          // measured projections in storage type
    void *d_ratio = nullptr;         // forward output / ratio in storage type
    float *d_vol32 = nullptr;        // float32 staging for host I/O
    float *d_proj32 = nullptr;
    double *d_sens = nullptr;        // A^T 1 in FP64 (EXACT)
    bool sens_valid = false;
    int32_t *d_shift = nullptr;      // shift-and-add table [nz][P]

    // launch tuning (set by kv_plan_autotune or defaults)
    int fwd_by = 4;                  // forward block = 32 x fwd_by rays
    int back_by = 8;                 // backprojector block = 32 x back_by voxels (one voxel per thread)
    int back_rows = 8;               // voxel rows per thread of the gather backprojector (0: one voxel per thread)
    int back_slices = 1;             // slices per thread of the gather backprojector

    // captured iteration loop (kv_mlem / kv_sart without callback), reused
    // while the buffers and parameters are the same
    cudaGraphExec_t graph_exec = nullptr;
    const void *graph_p = nullptr;
    const void *graph_x = nullptr;
    int graph_iters = 0, graph_mlem = 0, graph_fb = 0, graph_bb = 0;
    long long graph_slab = 0;
    int graph_br = 0, graph_bs = 0, graph_bst = 0;
    float graph_relax = 0.f;
};

// Drops one reference a plan (or network) held on its context; frees the
// context when it was destroyed by its owner and this was the last one.
void kv_ctx_release_ref(kv_ctx *ctx);

kv_status exact_batch_mlem_launch(kv_ctx *ctx, int n, kv_plan *const *plans, const float *const *p,
                                  float *const *x, int iters, float relax, int by, int bb);
kv_status exact_autotune(kv_plan *plan);

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------

kv_status kv_fail(kv_ctx *ctx, kv_status s, const char *fmt, ...);

#define KV_CHECK_CUDA(ctx, call)                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return kv_fail((ctx), e_ == cudaErrorMemoryAllocation ? KV_ERR_OOM : KV_ERR_CUDA, \
                           "%s failed: %s", #call, cudaGetErrorString(e_));                 \
    } while (0)

#define KV_CHECK_LAUNCH(ctx, what)                                                          \
    do {                                                                                    \
        cudaError_t e_ = cudaGetLastError();                                                \
        if (e_ != cudaSuccess)                                                              \
            return kv_fail((ctx), KV_ERR_CUDA, "%s launch failed: %s", what,                \
                           cudaGetErrorString(e_));                                         \
    } while (0)

#define KV_TRY(expr)                                                                        \
    do {                                                                                    \
        kv_status s_ = (expr);                                                              \
        if (s_ != KV_OK) return s_;                                                         \
    } while (0)

// ---------------------------------------------------------------------------
// Storage types
// ---------------------------------------------------------------------------

template <typename T> struct Store;
template <> struct Store<float> {
    static __device__ __forceinline__ float ld(const float *p) { return __ldg(p); }
    static __device__ __forceinline__ float ld_rw(const float *p) { return *p; }
    static __device__ __forceinline__ void st(float *p, float v) { *p = v; }
};
template <> struct Store<__nv_bfloat16> {
    static __device__ __forceinline__ float ld(const __nv_bfloat16 *p) {
        return __bfloat162float(__ldg(p));
    }
    static __device__ __forceinline__ float ld_rw(const __nv_bfloat16 *p) {
        return __bfloat162float(*p);
    }
    static __device__ __forceinline__ void st(__nv_bfloat16 *p, float v) {
        *p = __float2bfloat16_rn(v);
    }
};
template <> struct Store<__half> {
    static __device__ __forceinline__ float ld(const __half *p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float ld_rw(const __half *p) { return __half2float(*p); }
    static __device__ __forceinline__ void st(__half *p, float v) { *p = __float2half_rn(v); }
};

inline size_t kv_storage_bytes(kv_storage s) { return s == KV_STORAGE_F32 ? 4 : 2; }

// ---------------------------------------------------------------------------
// Kernel launchers (defined in the .cu files)
// ---------------------------------------------------------------------------

// Epilogue modes of the EXACT forward projector.
enum FwdMode : int {
    FWD_PLAIN = 0,    // out = A x
    FWD_MLEM = 1,     // out = Ls * (q > 0 ? relax * p / q : 0)      (pre-scaled ratio)
    FWD_SART = 2,     // out = Ls * (rowsum > 0 ? (p - q) / rowsum : 0)
    FWD_RESID = 3     // no output; FP64 residual / log-likelihood only
};
// Epilogue modes of the EXACT backprojector.
enum BackMode : int {
    BACK_PLAIN = 0,   // vol = A^T y'                  (y' already scaled by Ls)
    BACK_MLEM = 1,    // x = sens > 0 ? x * b / sens : x
    BACK_SART = 2     // x = sens > 0 ? x + relax * b / sens : x
};

struct FwdArgs {
    const void *vol;       // VolT [nz][ny][nx]
    const void *meas;      // ProjT measured projections (MLEM / SART / RESID)
    void *out;             // ProjT [P][nv][nu]
    double *red;           // FP64 reductions {sum (q-p)^2, sum p^2, sum p log q - q} or null
    float relax;
};
struct BackArgs {
    const void *yp;        // ProjT [P][nv][nu], scaled by the ray factor Ls
    void *vol;             // VolT output / iterate
    const double *sens;    // A^T 1 (MLEM / SART)
    float relax;
};

kv_status exact_build_tables(kv_plan *plan, const float *src, const float *det, int n_views,
                             ExactTables *out, ExactHostTables *host);
void exact_free_tables(ExactTables *t);

kv_status exact_forward_launch(kv_plan *plan, const ExactTables &t, int n_views, FwdMode mode,
                               const FwdArgs &a);
kv_status exact_back_launch(kv_plan *plan, BackMode mode, const BackArgs &a);
// The same launches restricted to views [v0, v0 + n) (forward, no reduction)
// and to slices [z0, z0 + nzs) (backprojection); per ray and per voxel the
// arithmetic is that of the whole launch.
kv_status exact_forward_views_launch(kv_plan *plan, int v0, int n, FwdMode mode, const FwdArgs &a);
kv_status exact_back_slab_launch(kv_plan *plan, BackMode mode, const BackArgs &a, int z0, int nzs);
kv_status exact_sensitivity_launch(kv_plan *plan, double *sens);
kv_status exact_prescale_launch(kv_plan *plan, const float *y, void *yp);

kv_status rc_forward_launch(kv_plan *plan, const float *d_src, const float *d_org, int n_views,
                            int mode, const float *vol, const float *meas, float *out,
                            float relax);
kv_status rc_back_launch(kv_plan *plan, int mode, const float *proj, float *vol);
// slices [z0, z0 + nzs) only; per voxel the arithmetic of the whole launch
kv_status rc_back_slab_launch(kv_plan *plan, int mode, const float *proj, float *vol, int z0, int nzs);

// shift-and-add; h_shift: the host copy of the [nz][P] shift table in d_shift
kv_status saa_launch(kv_plan *plan, const int32_t *d_shift, const int32_t *h_shift, const float *proj, float *out);
kv_status ramp_filter_launch(kv_plan *plan, const float *in, float *out, int half_taps);
kv_status fill_launch(kv_ctx *ctx, float *p, size_t n, float v);
kv_status convert_launch(kv_ctx *ctx, const float *in, void *out, size_t n, kv_storage s);
kv_status convert_back_launch(kv_ctx *ctx, const void *in, float *out, size_t n, kv_storage s);
kv_status phantom_launch(kv_ctx *ctx, int nx, int ny, int nz, float dx, float dy, float dz,
                         const float *d_params, int n, float *vol);

// Slab-staged EXACT forward projector (kv_fwd_slab.cu).  fwd_slab_fit checks
// that the plan's geometry suits it (at most three columns and five rows per
// ray and slice, boxes within 256 voxels and the shared-memory budget) and
// sizes its boxes for (R, S, stages, group); fwd_slab_launch runs it for
// views [0, n_views) of the tables `t` (the plan's own, possibly offset).
bool fwd_slab_fit(const kv_plan *plan, int R, int S, int stages, int group, FwdSlabCfg *out, std::string *why);
int fwd_slab_default_group(int n_views);
size_t fwd_slab_blocks(const kv_plan *plan, int n_views);
kv_status fwd_slab_launch(kv_plan *plan, const ExactTables &t, int n_views, FwdMode mode, const FwdArgs &a,
                          double *partials);

// TMA-staged EXACT backprojector (kv_back_stage.cu): back_stage_fit checks
// that the plan suits it (FP32 storage, 16-byte detector rows, every
// voxel tile's view of the detector within 256 x 256 pixels and the
// shared-memory budget) and sizes the patch for (R, stages);
// back_stage_launch runs slices [z0, z0 + nzs) over the plan's first n_views
// views (all of them outside the autotuner).
bool back_stage_fit(const kv_plan *plan, int R, int stages, BackStageCfg *out, std::string *why);
kv_status back_stage_launch(kv_plan *plan, BackMode mode, const BackArgs &a, int z0, int nzs, int n_views);

// RC driver epilogue modes (forward: ratio / residual fused; back: update fused)
enum RcMode : int { RC_PLAIN = 0, RC_MLEM = 1, RC_ART = 2 };
