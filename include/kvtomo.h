/*
 * kvtomo.h -- C ABI of the GB300 tomosynthesis projector / reconstruction engine.
 *
 * Every entry point is plain C: opaque handles, POD structs, raw pointers and
 * sizes, a kv_status return code.  Nothing here exits the process; a failing
 * call returns a status and kv_ctx_last_error() gives the message.
 *
 * Reference interfaces replaced (paths inside the Kevernals project):
 *   kv_forward        <- Projector::PerformProjection(ImageDataPtr)
 *                        source/modules/reconstruction/Projector.cu:873-1036
 *                        (kernel CudaPerformProjection, Projector.cu:227-372)
 *   kv_forward_single <- Projector::PerformProjection(volume, Position3D, container)
 *                        Projector.cu:823-870 (left unfinished in the reference)
 *   kv_back           <- Projector::PerformBackProjection(ImageDataPtr)
 *                        Projector.cu:1038-1207 (kernel Projector.cu:376-785),
 *                        recons::BackProjection Reconstructors.h:256-261
 *   kv_sart           <- recons::ART      Reconstructors.h:19-134
 *   kv_mlem           <- recons::MLEM     Reconstructors.h:136-253
 *   kv_shift_and_add  <- recons::ShiftAndAdd Reconstructors.h:263-379
 *   kv_geometry       <- the arrays Projector.cu:917-940 flattens out of
 *                        TomoGeometry (TomoGeometry.h:34-89)
 *   kv_uniform_volume <- PhantomMaker(volume, 1.f).GetPhantom(), the uniform
 *                        start of ART/MLEM (Reconstructors.h:35-36, 152-153)
 * Entry points without a reference counterpart (sensitivity image, FP64
 * residual reductions, batched solves) say so beside their declaration.
 *
 * Conventions
 *   Frame: volume-centred, as in the reference (TomoGeometry.cpp:127,162,330).
 *   Volume: float32 [nz][ny][nx], x fastest; voxel (i,j,k) spans
 *           [-nx*dx/2 + i*dx, -nx*dx/2 + (i+1)*dx] (same for y, z).
 *   Projections: float32 [n_views][nv][nu], u fastest; pixel (u,v) of view p
 *           has its centre at det_origin[p] + ((u+0.5)*du, (v+0.5)*dv, 0).
 *   Memory: each data call takes a kv_mem flag.  KV_MEM_HOST: the library
 *           copies in and out (pinned staging, stream-ordered, synchronous on
 *           return).  KV_MEM_DEVICE: pointers are device memory of the
 *           context's device; the call is asynchronous on the context stream.
 *           The library never frees caller memory.
 *   Threading: one kv_ctx per host thread; calls on a context are ordered on
 *           its stream.
 */
#ifndef KVTOMO_H
#define KVTOMO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KV_ABI_VERSION 1

typedef enum kv_status {
    KV_OK = 0,
    KV_ERR_INVALID_ARG = 1, /* null pointer, size out of range, bad enum          */
    KV_ERR_GEOMETRY = 2,    /* geometry the chosen operator family cannot express  */
    KV_ERR_OOM = 3,         /* device or pinned host allocation failed             */
    KV_ERR_CUDA = 4,        /* a CUDA runtime call failed                          */
    KV_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up                  */
    KV_ERR_NUMERIC = 6,     /* non-finite input or result                          */
    KV_ERR_UNSUPPORTED = 7, /* operation not defined for this family / storage     */
    KV_ERR_NO_DEVICE = 8    /* no CUDA device, or the device is not sm_103         */
} kv_status;

/* Operator family.
 * KV_FAMILY_RC reproduces the reference kernels, quirks included: the forward
 *   value of a ray is the path-length weighted MEAN of the voxels it crosses
 *   (Projector.cu:348-371) and the backprojection is the voxel-driven,
 *   11x11-window, weight-normalised operator (Projector.cu:452-776).
 * KV_FAMILY_EXACT is the Siddon line integral A (mm * value) and its exact
 *   transpose A^T; it needs the detector plane below the volume and every
 *   source above it (the linear-sweep tomosynthesis geometry). */
typedef enum kv_family { KV_FAMILY_RC = 0, KV_FAMILY_EXACT = 1 } kv_family;

/* Storage type of the volume and projections while a solve runs on the
 * device.  Arithmetic is FP32 in every case; the API buffers stay float32. */
typedef enum kv_storage { KV_STORAGE_F32 = 0, KV_STORAGE_BF16 = 1, KV_STORAGE_F16 = 2 } kv_storage;

typedef enum kv_mem { KV_MEM_HOST = 0, KV_MEM_DEVICE = 1 } kv_mem;

typedef struct kv_geometry {
    int32_t nx, ny, nz;       /* volume size in voxels                                  */
    float dx, dy, dz;         /* voxel spacing (mm)                                     */
    int32_t n_views;          /* number of projections                                  */
    int32_t nu, nv;           /* detector ROI size in pixels                            */
    float du, dv;             /* detector pixel spacing (mm)                            */
    const float *src;         /* [n_views][3] source positions                          */
    const float *det_origin;  /* [n_views][3] ROI bottom-left corner; z = detector plane */
    float fulcrum_z;          /* shift-and-add focal height (TomoGeometry::fulcrum().z)   */
} kv_geometry;

typedef struct kv_ctx kv_ctx;
typedef struct kv_plan kv_plan;

/* Per-iteration callback of the iterative drivers.  residual is
 * ||A x - p||_2 / ||p||_2 of the iterate entering the iteration and loglik the
 * Poisson log-likelihood sum(p log(Ax) - Ax), both reduced in FP64; they are
 * only computed when a callback is given.  Return nonzero to stop early. */
typedef int (*kv_iter_cb)(int iteration, double residual, double loglik, void *user);

/* ---- library / context ------------------------------------------------ */
/* No reference counterpart as functions: the reference uses the CUDA
 * default device and stream implicitly and exits on a CUDA error
 * (checkCudaErrors, CudaErrorHandler.h:581-594).  A context makes the
 * device and stream explicit; kv_status, kv_status_string and
 * kv_ctx_last_error replace that exit (and play the part of the
 * Result<T> / std::error_code convention, Result.h:17-41). */
const char *kv_version(void);
const char *kv_status_string(kv_status s);
kv_status kv_ctx_create(int device, kv_ctx **out);
kv_status kv_ctx_destroy(kv_ctx *ctx);
/* Use `stream` (a cudaStream_t of the context's device; NULL is the CUDA
 * default stream) for every later call on this context.  A new context uses a
 * stream of its own. */
kv_status kv_ctx_set_stream(kv_ctx *ctx, void *cuda_stream);
kv_status kv_sync(kv_ctx *ctx);
const char *kv_ctx_last_error(const kv_ctx *ctx);
/* Tracing (no reference counterpart: the reference prints grid sizes and the
 * last CUDA error, Projector.cu:948-962).  While enabled, every kernel the
 * context launches is bracketed by CUDA events on its stream.
 * kv_ctx_timing_read synchronises the stream and writes one line per kernel
 * name, "<name> <launches> <total device ms>", into buf (NUL-terminated,
 * truncated to buflen), then clears the records. */
kv_status kv_ctx_set_timing(kv_ctx *ctx, int enable);
kv_status kv_ctx_timing_read(kv_ctx *ctx, char *buf, size_t buflen);

/* ---- plans -------------------------------------------------------------- */
/* Validates the geometry, uploads per-view tables, and keeps the workspace a
 * solve needs.  The geometry arrays are copied; the caller may free them.
 * Replaces the geometry flattening and device set-up that
 * Projector::PerformProjection / PerformBackProjection repeat on every call
 * (Projector.cu:873-954, 1038-1125): here they are done once per plan. */
kv_status kv_plan_create(kv_ctx *ctx, const kv_geometry *geom, kv_family family,
                         kv_storage storage, kv_plan **out);
kv_status kv_plan_destroy(kv_plan *plan);
/* Number of elements of the volume and of the projection stack. */
size_t kv_plan_volume_elems(const kv_plan *plan);
size_t kv_plan_proj_elems(const kv_plan *plan);

/* ---- operators ---------------------------------------------------------- */
kv_status kv_forward(kv_plan *plan, const float *volume, float *projections, kv_mem mem);
/* Forward projection of one view (source position and detector origin given
 * explicitly) into an nv x nu container; completes Projector.cu:823-870. */
kv_status kv_forward_single(kv_plan *plan, const float *volume, const float src[3],
                            const float det_origin[3], float *projection, kv_mem mem);
kv_status kv_back(kv_plan *plan, const float *projections, float *volume, kv_mem mem);
/* Sensitivity image A^T 1, accumulated in FP64 (EXACT only).  No reference
 * counterpart: the reference MLEM normalises inside its backprojector. */
kv_status kv_sensitivity(kv_plan *plan, double *sens, kv_mem mem);
/* Shift-and-add tomosynthesis: [nz][nv][nu] slices, one per volume slice, the
 * detector ROI size as in the reference.  RC uses the reference's shift rule
 * literally (Reconstructors.h:308-331); EXACT measures heights from the
 * detector plane and shifts in detector pixels. */
kv_status kv_shift_and_add(kv_plan *plan, const float *projections, float *slices, kv_mem mem);
/* Filtered backprojection for tomosynthesis (EXACT family, FP32 storage):
 *   volume = A^T(h * p) / A^T 1   (0 where A^T 1 = 0)
 * where h * p filters every detector column along v, the tube's sweep
 * direction, with the Shepp-Logan ramp kernel h[n] = -2 / (pi^2 (4n^2 - 1))
 * (pixel units) truncated at |n| <= half_taps (1..KV_FBP_MAX_HALF_TAPS),
 * zero outside the detector.  A sharpened shift-and-add: the same
 * normalisation as one SART step from zero, with ramp-filtered data.  The
 * reference's "FBP" reconstructor is an unfiltered backprojection
 * (backup/TomosynthesisFBPReconstructor.cpp); this is the filtered method. */
#define KV_FBP_MAX_HALF_TAPS 256
kv_status kv_fbp(kv_plan *plan, const float *projections, float *volume, int32_t half_taps, kv_mem mem);
/* Host-only: the integer row shift of every (slice, view) pair that
 * kv_shift_and_add applies, [nz][n_views], computed without a device.
 * Replaces the shift loop of recons::ShiftAndAdd, Reconstructors.h:308-331.
 * Values are the rule's own, limited to +-2^30; non-finite geometry values
 * are refused (KV_ERR_INVALID_ARG / KV_ERR_NUMERIC). */
kv_status kv_shift_and_add_shifts(const kv_geometry *geom, kv_family family, int32_t *shifts);
/* Fill `volume` with the uniform initial estimate 1.0 (PhantomMaker(vol,1.f)). */
kv_status kv_uniform_volume(kv_plan *plan, float *volume, kv_mem mem);

/* Rasterises a sum of ellipsoids, sampled at voxel centres, into a volume of
 * nx*ny*nz voxels centred at the origin.  params holds n rows of 16 floats:
 * centre[3], semi-axes[3], M[9] (row-major, local coordinates = M (q - c)),
 * density.  Used to generate seeded phantoms for the benchmarks and the
 * warm-start training data.  No reference counterpart: the reference phantom
 * (PhantomMaker.cpp:9-51) has boxes and spheres sampled at voxel corners. */
kv_status kv_phantom_ellipsoids(kv_ctx *ctx, int32_t nx, int32_t ny, int32_t nz, float dx, float dy,
                                float dz, const float *params, int32_t n, float *volume, kv_mem mem);

/* ---- iterative drivers -------------------------------------------------- */
/* MLEM.  RC: q = A x; where q != 0, q <- relax * p / q; x <- x * B(q), the
 * reference semantics.  EXACT: x <- x * A^T(relax * p / A x) / A^T 1.  The
 * volume is updated in place, as the reference does with its initial volume.
 * With KV_MEM_HOST buffers (FP32 storage, no callback) the uploads and the
 * final download overlap the first forward projection and the last
 * backprojection on an internal copy stream; the call still returns only
 * when the volume is back in host memory, and the result equals the
 * KV_MEM_DEVICE call bit for bit. */
kv_status kv_mlem(kv_plan *plan, const float *projections, float *volume_inout, int iterations,
                  float relax, kv_mem mem, kv_iter_cb cb, void *user);
/* Simultaneous ART.  RC: x <- x + B(relax * (p - A x)) (recons::ART).  EXACT:
 * SART, x <- x + relax * C A^T(R (p - A x)), R = 1/(A 1), C = 1/(A^T 1). */
kv_status kv_sart(kv_plan *plan, const float *projections, float *volume_inout, int iterations,
                  float relax, kv_mem mem, kv_iter_cb cb, void *user);
/* Batched MLEM: n independent EXACT/FP32 reconstructions of uneven volume,
 * detector and view counts, all created on `ctx`, run together.  Each
 * iteration is one persistent forward launch and one persistent
 * backprojection launch over the tiles of every problem; the whole
 * `iterations` loop is captured as one CUDA graph.  Results are identical to
 * calling kv_mlem on each plan.  No reference counterpart (the reference
 * reconstructs one case per call).  projections[i] / volumes[i] are host or
 * device buffers according to `mem`; volumes are updated in place. */
kv_status kv_batch_mlem(kv_ctx *ctx, int n, kv_plan *const *plans, const float *const *projections,
                        float *const *volumes, int iterations, float relax, kv_mem mem);

/* Autotuner (no reference counterpart; the reference launches every kernel
 * with a fixed 32x16 block).  On (a subset of the views of) this plan's
 * geometry it times the slab forward projector's shapes (rays per thread,
 * slices per slab, stages: see kv_plan_set_slab), the gather
 * backprojector's shapes (kv_plan_set_back_shape, including one voxel per
 * thread) and the one-thread-per-ray / per-voxel kernels' block heights
 * (32 x {1,2,4,8} rays, 32 x {2,4,8} voxels), each the median of three
 * timed runs, and keeps the fastest; results are cached per geometry shape
 * and storage for the process.  kv_plan_get_tuning reports the block
 * heights. */
kv_status kv_plan_autotune(kv_plan *plan);
kv_status kv_plan_get_tuning(const kv_plan *plan, int *fwd_rows, int *back_rows);
kv_status kv_plan_set_tuning(kv_plan *plan, int fwd_rows, int back_rows);

/* Shape of the slab-staged EXACT forward projector (no reference
 * counterpart; it replaces the per-pixel-thread CudaPerformProjection,
 * Projector.cu:227-372, on the EXACT path): CTAs of 32 x 8*rays_per_thread
 * detector rays, the volume staged `slices` slices at a time in shared
 * memory with `stages` slabs in flight, `view_group` consecutive views
 * launched together.  rays_per_thread = 0 selects the one-thread-per-ray
 * kernel.  Plans take a default shape when their geometry suits it (at most
 * two column and four row planes crossed per ray and slice); set returns
 * KV_ERR_UNSUPPORTED with a reason when a shape does not fit the geometry.
 * get reports rays_per_thread = 0 when the plan runs the per-ray kernel. */
kv_status kv_plan_get_slab(const kv_plan *plan, int *rays_per_thread, int *slices, int *stages, int *view_group);
kv_status kv_plan_set_slab(kv_plan *plan, int rays_per_thread, int slices, int stages, int view_group);

/* Work per thread of the EXACT gather backprojector (no reference
 * counterpart; it replaces the per-voxel-thread CudaPerformBackProjection,
 * Projector.cu:376-785, on the EXACT path): voxel rows per thread share each
 * thread's candidate-column intervals, and consecutive slices per thread
 * are summed view by view so that they reuse each view's detector patch
 * from cache.  Shapes (rows, slices): (1, 1), (2, 1), (2, 2), (4, 1),
 * (4, 2), (8, 1); all give bit-identical volumes.  Rows 0 selects
 * one voxel per thread in blocks of 32 x back_rows of kv_plan_set_tuning.
 * Default (8, 1). */
kv_status kv_plan_get_back_shape(const kv_plan *plan, int *rows_per_thread, int *slices_per_thread);
kv_status kv_plan_set_back_shape(kv_plan *plan, int rows_per_thread, int slices_per_thread);

/* The EXACT backprojector with each view's detector patch staged in shared
 * memory by TMA, one view ahead (no reference counterpart; it replaces the
 * gather kernels of kv_plan_set_back_shape for FP32 storage when set): 4 or
 * 8 voxel rows per thread, 2 or 3 stages; rows 0 turns it off.  Its volumes
 * are bit-identical to the gather kernels'.  KV_ERR_UNSUPPORTED when the
 * plan does not suit it (16-bit storage, detector rows that are not a whole
 * number of 16 bytes, a voxel tile that sees more than 256 x 256 detector
 * pixels, or patches beyond the shared-memory budget).  The getter also
 * reports the patch size in detector columns and rows. */
kv_status kv_plan_get_back_staging(const kv_plan *plan, int *rows_per_thread, int *stages, int *patch_cols,
                                   int *patch_rows);
kv_status kv_plan_set_back_staging(kv_plan *plan, int rows_per_thread, int stages);

/* ---- learned warm start (no reference counterpart) ----------------------
 * A 3D U-Net (4 levels, 16/32/64/128 channels, 3x3x3 convolutions, BF16
 * weights and activations, FP32 accumulation, tensor-core implicit-GEMM
 * convolutions) mapping a shift-and-add volume [D][H][W] (float32) to an MLEM
 * initial estimate of the same size: y = x + f(x).  D and H must be multiples
 * of 8 and W of 128. */
/* One of the network's convolutions on caller device buffers: out =
 * conv3x3x3(in1 ++ in2, w) + bias, ReLU if relu != 0, zero padding.
 * Channels-last BF16 (bit patterns) [D][H][W][C]: in1 has c1 channels, in2
 * (may be NULL when c2 = 0) c2 channels concatenated after them, out cout
 * channels; w is [cout][27][c1 + c2] BF16 (taps z, y, x), bias cout floats
 * or NULL; FP32 accumulation.  kernel: 0 = tcgen05 / TMA implicit GEMM where
 * the volume is a whole number of 128-voxel tiles, else mma.sync; 1 =
 * tcgen05 only; 2 = mma.sync only.  Channel counts: multiples of 16 (the
 * tcgen05 kernel: 16, 32, 64 or 128 per input, cout <= 256).  Stream-ordered
 * on the context's stream; a tensor-core pipeline wait that gives up is
 * reported by the next kv_sync. */
kv_status kv_conv3_bf16(kv_ctx *ctx, const uint16_t *in1, int32_t c1, const uint16_t *in2, int32_t c2,
                        const uint16_t *w, const float *bias, int32_t relu, uint16_t *out, int32_t cout,
                        int32_t D, int32_t H, int32_t W, int32_t kernel);

/* The learned warm start's elementwise steps on device buffers of n
 * elements, on the context's stream (no reference counterpart).
 *   kv_warm_ratio      ratio = a1 > 0 ? p / a1 : 0 -- the ray ratio of the
 *                      volume-grid shift-and-add A^T(p / A1) / A^T 1 -- and,
 *                      if uniform_residual is not NULL, ||a1 - p|| / ||p|| in
 *                      FP64: the data residual of the uniform start, whose
 *                      projection is the ray-length image a1 (synchronises).
 *   kv_warm_normalize  out = sens > 0 ? b / sens : 0, divided in FP64.
 *   kv_warm_fill       out = max(seen ? net : saa, eps): the network's
 *                      estimate with the voxels no ray sees enough of taken
 *                      from the shift-and-add volume, clamped positive. */
kv_status kv_warm_ratio(kv_ctx *ctx, const float *p, const float *a1, float *ratio, size_t n,
                        double *uniform_residual);
kv_status kv_warm_normalize(kv_ctx *ctx, const float *b, const double *sens, float *out, size_t n);
kv_status kv_warm_fill(kv_ctx *ctx, const float *net, const float *saa, const uint8_t *seen, float eps,
                       float *out, size_t n);

typedef struct kv_unet kv_unet;
kv_status kv_unet_create(kv_ctx *ctx, uint64_t seed, kv_unet **out);
kv_status kv_unet_destroy(kv_unet *net);
size_t kv_unet_num_params(const kv_unet *net);
kv_status kv_unet_forward(kv_unet *net, const float *in, float *out, int32_t D, int32_t H, int32_t W,
                          kv_mem mem);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on the mean squared error
 * between net(in) and target; *loss is the loss before the step.  Target
 * voxels that are NaN carry no target: they add nothing to the loss (which
 * stays a sum over the other voxels divided by D*H*W). */
kv_status kv_unet_train_step(kv_unet *net, const float *in, const float *target, int32_t D, int32_t H,
                             int32_t W, float lr, float *loss, kv_mem mem);
/* Loss and FP32 parameter gradients (host buffer of kv_unet_num_params). */
kv_status kv_unet_gradients(kv_unet *net, const float *in, const float *target, int32_t D, int32_t H,
                            int32_t W, float *loss, float *grads, kv_mem mem);
/* Checkpoint state: parameters, Adam moments (3 * num_params host floats) and
 * the step count. */
kv_status kv_unet_get_state(const kv_unet *net, float *state, int64_t *step);
kv_status kv_unet_set_state(kv_unet *net, const float *state, int64_t step);

/* ||A x - p||_2 / ||p||_2 and sum(p log(Ax) - Ax) reduced in FP64.  No
 * reference counterpart (the reference has no stopping criterion). */
kv_status kv_residual(kv_plan *plan, const float *projections, const float *volume, kv_mem mem,
                      double *rel_residual, double *loglik);

/* The same FP64 residual and log-likelihood as kv_residual, computed without
 * allocating any device memory.  No reference counterpart.  For callers that
 * may not allocate when they need a residual: real-time loops that must not
 * touch the allocator, or hosts whose device memory is owned by another
 * framework's allocator or a fixed budget.  The plan (created beforehand) must
 * be KV_FAMILY_EXACT with KV_STORAGE_F32; `projections` and `volume` are
 * device pointers; the results are written to the two host doubles.
 * Scratch: a static device array of KV_NOALLOC_MAX_BLOCKS FP64 partial-sum
 * triples (1.5 MiB) that every GPU loading the library holds until the
 * process exits.  The residual runs the one-thread-per-ray forward kernel in
 * blocks of 32 x fwd_rows rays, fwd_rows being the plan's forward block
 * height (kv_plan_get_tuning: 4 unless kv_plan_set_tuning or
 * kv_plan_autotune changed it, at most 8); a geometry with
 *     ceil(nu / 32) * ceil(nv / fwd_rows) * n_views > KV_NOALLOC_MAX_BLOCKS
 * is rejected with KV_ERR_INVALID_ARG -- use kv_residual for it.  The first
 * call on a device looks up the array's device address and keeps it for the
 * life of that device's primary context (do not call this entry point again
 * after resetting the device in the same process); make that first call
 * before any stream capture.  The call leaves the caller's current device as
 * it found it.  All calls share the array: calls that overlap on one GPU race
 * and must be serialised by the caller. */
#define KV_NOALLOC_MAX_BLOCKS 65536
kv_status kv_residual_noalloc(kv_plan *plan, const float *projections, const float *volume,
                              double *rel_residual, double *loglik);

#ifdef __cplusplus
}
#endif
#endif /* KVTOMO_H */
