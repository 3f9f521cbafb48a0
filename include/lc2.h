/*
 * lc2.h -- C ABI of the GB300 LC2 similarity library (liblc2.so).
 *
 * Drop-in boundary for the similarity hot path of LC2Registration. The
 * reference exposes C++ classes, not a C ABI; each entry point below names
 * the reference interface it replaces (paths relative to the reference
 * project root). All entry points return an lc2_status (0 = success); the
 * message of the last failure on the calling thread is lc2_last_error().
 *
 * Conventions:
 *   - images/volumes are float32, x fastest (index x + y*X + z*X*Y), the
 *     reference's layout; 2D images use dim[2] = 1;
 *   - transforms are row-major virtual->moving mm matrices: 3x3 (9 floats)
 *     in 2D mode, 4x4 (16 floats) in 3D and 2D-to-3D modes -- the matrix
 *     the reference uploads as VirtualToMoving{2,3}D_d
 *     (src/Interpolator/interpolator.cuh:32-41);
 *   - a context owns its device memory and one CUDA stream; there is no
 *     process-global state, so contexts are independent and thread-safe
 *     per context (the reference keeps geometry in process-global
 *     __constant__ symbols, src/Interpolator/interpolator.cuh:27-41).
 */
#ifndef LC2_H
#define LC2_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    LC2_OK = 0,
    LC2_ERR_INVALID_ARGUMENT = 1, /* bad dims, patch size, null pointer, NaN/Inf input */
    LC2_ERR_OUT_OF_MEMORY = 2,    /* device or host allocation failed */
    LC2_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    LC2_ERR_NOT_READY = 4,        /* images not set yet */
    LC2_ERR_SINGULAR = 5,         /* non-invertible transform */
    LC2_ERR_UNSUPPORTED = 6,      /* mode/patch size outside the supported range */
    LC2_ERR_TIMEOUT = 7           /* a bounded device-side wait expired; the context
                                     stays usable */
} lc2_status;

typedef enum { LC2_MODE_2D = 0, LC2_MODE_3D = 1, LC2_MODE_2DTO3D = 2 } lc2_mode;

/* Storage type of the gathered (moving) volume and of the static ultrasound
 * image on the device; arithmetic is FP32/integer regardless. */
typedef enum { LC2_STORE_F32 = 0, LC2_STORE_F16 = 1, LC2_STORE_BF16 = 2 } lc2_storage;

typedef struct {
    int dim[3];        /* voxels; 2D images: dim[2] = 1 */
    float spacing[3];  /* mm */
    float origin[3];   /* mm */
} lc2_geometry;

typedef struct {
    int mode;                /* lc2_mode */
    lc2_geometry fixed;      /* FixedImage / FixedVolume */
    lc2_geometry moving;     /* MovingImage / MovingVolume */
    float virtual_spacing[3];/* RegistrationParameters.ResampledSpacing */
    int patch_size;          /* RegistrationParameters.PatchSize (radius r, patch 2r+1);
                              * 0 = normalised mutual information (3D) */
    int high_res_is_moving;  /* HighResolutionModality: 1 = Moving, 0 = Fixed */
    int storage;             /* lc2_storage */
    int max_batch;           /* transforms per launch group of the generic kernels
                              * (LC2_OPTION_GENERIC; each holds one warped image of
                              * scratch); 0 = one. The fused kernels take any batch
                              * in one launch. */
    int device;              /* CUDA device ordinal */
} lc2_config;

typedef struct lc2_context lc2_context;

/* Creates a context: virtual grid, device buffers, stream.
 * Replaces Interpolator{2D,3D,2DTo3D}::Interpolator{...}(const LC2Configuration*)
 * + InitiateMappers + InitiateRegistrationHandle
 * (src/Interpolator/interpolator.cu:393-529, :1105-1246, :1538-1676) and
 * LC2_{2D,3D}_class::PortedFromInterpolator (src/cu_LC2/cu_lc2_2d.cu:515-546,
 * src/cu_LC2/cu_lc2_3d.cu:942-975). */
int lc2_create(const lc2_config* cfg, lc2_context** out);

/* Releases all device memory and the stream of the context. */
int lc2_destroy(lc2_context* ctx);

/* Uploads fixed and moving images (host float32) and precomputes the
 * static virtual-grid image. Replaces the FixedVolume_d / MovingVolume_d
 * uploads (src/Interpolator/interpolator.cu:276,315,459-473). */
int lc2_set_images(lc2_context* ctx, const float* fixed_host, const float* moving_host);

/* lc2_set_images for images that are already in device memory of the
 * context's device (float32, same layout): the buffers the reference's
 * LC2_{2D,3D}_class hold as thrust::device_vector and fill on the device
 * (src/cu_LC2/cu_lc2_3d.cuh:75-89, src/cu_LC2/cu_lc2_2d.cuh:55-66). The
 * inputs are read, not kept: later changes to them need another call.
 * Host pointers are refused with LC2_ERR_INVALID_ARGUMENT. */
int lc2_set_images_device(lc2_context* ctx, const float* fixed_device,
                          const float* moving_device);

/* The configuration the context was created with. */
int lc2_get_config(const lc2_context* ctx, lc2_config* out);

/* Virtual grid dims (src/Interpolator/interpolator.cu:337-339). */
int lc2_virtual_dims(const lc2_context* ctx, int dims[3]);

/* One LC2 evaluation for one transform (the plain form). Replaces the
 * per-objective sequence GenerateMappers -> Interpolate ->
 * GetSimilarityMeasure (src/Optimizers/optimizers.cu:170-176,702-707;
 * src/Interpolator/interpolator.cu:542-631; src/cu_LC2/cu_lc2_3d.cu:1119-1194).
 * *lc2_out = sum(measure)/sum(sigma), 0 when NaN/Inf. */
int lc2_evaluate(lc2_context* ctx, const float* matrix, double* lc2_out);

/* `count` evaluations (matrices packed back to back). Batched form of
 * lc2_evaluate; results are identical to `count` plain calls. */
int lc2_evaluate_batch(lc2_context* ctx, const float* matrices, int count, double* lc2_out);

/* Asynchronous pieces of lc2_evaluate_batch, for callers that time or
 * overlap the device work: stage copies the matrices to the device, launch
 * enqueues every kernel on the context stream, fetch copies results back and
 * synchronises the stream. */
int lc2_stage_transforms(lc2_context* ctx, const float* matrices, int count);
int lc2_launch_staged(lc2_context* ctx, int count);
int lc2_fetch_results(lc2_context* ctx, double* lc2_out, int count);

/* The context's CUDA stream (a cudaStream_t), and an override with a
 * caller-owned stream (NULL restores the context's own stream). */
void* lc2_get_stream(const lc2_context* ctx);
int lc2_set_stream(lc2_context* ctx, void* stream);

/* Diagnostic evaluation that also downloads the per-voxel virtual-grid
 * fields (any pointer may be NULL): ultrasound U, high-resolution image M,
 * its Sobel magnitude G, weighting factor sigma and clipped measure.
 * Mirrors the buffers behind LC2_{2D,3D}_class::Get*Buffer/Get*RawPointer
 * (src/cu_LC2/cu_lc2_2d.cu:821-831, src/cu_LC2/cu_lc2_3d.cu:1331-1345). */
int lc2_evaluate_fields(lc2_context* ctx, const float* matrix, double* lc2_out, float* U,
                        float* M, float* G, float* sigma, float* measure);

/* Weighting map of one evaluation: measure / sigma per virtual voxel, 0
 * where sigma is not above 1e-6 (LC2_3D_class::GenerateWeightingMap /
 * CalculateWeightingMap, src/cu_LC2/cu_lc2_3d.cu:843-866, 1303-1329; here
 * for 2D grids too). map: virtual-grid floats; *lc2_out (may be NULL) the
 * evaluation's LC2. */
int lc2_weighting_map(lc2_context* ctx, const float* matrix, double* lc2_out, float* map);

/* The registered 2D image: src (sw x sh) warped into dst (dw x dh) by the
 * forward pixel map (x', y') = C (x, y, 1), coeffs = C's two rows, bilinear,
 * destination pixels whose source falls outside src left at 0. Replaces the
 * nppiWarpAffine_32f_C1R call of Interpolator2D::WriteOut
 * (src/Interpolator/interpolator.cu:1438-1535). Host buffers; runs on
 * `device`. */
int lc2_warp_affine_2d(const float* src, int sw, int sh, float* dst, int dw, int dh,
                       const double coeffs[6], int device);

/* Kernel launches issued by this context since creation (device work
 * accounting for benchmarks). */
long long lc2_launch_count(const lc2_context* ctx);

/* Tuning options (lc2_set_option). LC2_OPTION_TILE_ROWS: output rows per
 * tile of the fused 3D kernels at patch radius 1-4: 16 (one 512-thread CTA
 * per SM), 24 (one 768-thread CTA per SM; on presampled images, and for a
 * resampled MR/CT resampled in the kernel; elsewhere taken as 16; a grid
 * whose height leaves 1-16 rows over runs them on 16-row tiles) or 8 (two
 * CTAs per SM); radius 5-6 always runs 8. 0 = automatic: 24 on presampled
 * images -- of a resampled MR/CT on any grid, of a resampled ultrasound on
 * grids of 8 M voxels or more -- and for a resampled MR/CT at radius 3 or 4
 * when the kernel resamples itself (LC2_OPTION_PRESAMPLE 0); else 16. 2D and
 * 2D-to-3D contexts with a resampled MR/CT: 16 or 32 (two 1024-thread CTAs
 * per SM, patch radius 4 to 6; other radii take it as 16); 0 = per launch
 * (32 where it exists and the launch has four CTAs per SM or more). No
 * counterpart in the reference (its block sizes are arguments of
 * CalculateGradient / GetSimilarityMetric, src/cu_LC2/cu_lc2_3d.cuh:36-41). */
enum { LC2_OPTION_TILE_ROWS = 1 };
/* LC2_OPTION_ZCHUNK: output slices each CTA of the fused 3D kernel marches
 * through (0 = automatic). LC2_OPTION_GRAPHS: 1 (default) replays
 * lc2_evaluate_batch / lc2_evaluate from a CUDA graph captured once per batch
 * size; 0 issues the calls one by one. None of these options changes a
 * result: every sum is exact, whatever the tiling. */
enum { LC2_OPTION_ZCHUNK = 2, LC2_OPTION_GRAPHS = 3 };
/* LC2_OPTION_PIPELINE: 1 runs 3D evaluations with patch radius <= 4 on the
 * warp-specialised fused kernel (producer warps resample the next slices
 * into a shared ring while consumer warps do the moments); 0 (default) the
 * single-role kernel. Same values either way. Every producer/consumer wait
 * of that kernel gives up after one second: the kernel then stops its CTA,
 * and the call that launched it (or the next lc2_fetch_results) returns
 * LC2_ERR_TIMEOUT with the context still usable. */
enum { LC2_OPTION_PIPELINE = 4 };
/* Self-test of that failure path: runs the same bounded wait, for one
 * second, on a barrier that nothing completes, on the context's stream.
 * Returns LC2_ERR_TIMEOUT when the wait expired and was reported as it must
 * (the expected result), LC2_OK if it did not expire; nothing faults, traps
 * or hangs, and the context's later evaluations are unaffected. No
 * counterpart in the reference (it checks no CUDA status at all). */
int lc2_wait_probe(lc2_context* ctx);
/* LC2_OPTION_STREAM_PRIORITY: recreates the context's own stream with this
 * CUDA stream priority (lower = more urgent, clamped to the device's range;
 * see cudaDeviceGetStreamPriorityRange). The server gives small requests the
 * most urgent priority so their launches are scheduled ahead of large ones. */
enum { LC2_OPTION_STREAM_PRIORITY = 5 };
/* LC2_OPTION_GENERIC: 1 evaluates through the generic kernels (resampling,
 * Sobel and patch moments as separate launches through global scratch)
 * instead of the fused kernel of the context's modality; for cross-checks.
 * The values agree to FP32 resampling rounding (the two paths place their
 * sampling bases differently). */
enum { LC2_OPTION_GENERIC = 7 };
/* LC2_OPTION_PRESAMPLE (3D, HighResolutionModality Moving): how the moving
 * image is resampled. 1 (the default of such contexts): in a pass of its own,
 * one float per virtual voxel and transform written to a context buffer that
 * grows with the batch up to 2 GiB (32 transforms at 256^3; larger batches
 * run in groups), which the fused kernel then reads; 0: inside the fused
 * kernel. Other values are refused (LC2_ERR_INVALID_ARGUMENT). Each voxel is
 * sampled once from its 32 x 8 tile's base in form 1 and from the fused
 * tile's base in form 0, so 0 and 1 agree to FP32 resampling rounding (about
 * 1e-7 relative on LC2), not bit for bit. Within a form no option changes a
 * value. */
enum { LC2_OPTION_PRESAMPLE = 8 };
int lc2_set_option(lc2_context* ctx, int option, int value);

/* CUDA-graph launches issued by lc2_evaluate_batch / lc2_evaluate. */
long long lc2_graph_launches(const lc2_context* ctx);

/* Autotuner: times the fused kernel on `count` transforms (matrices as in
 * lc2_evaluate_batch) for each tile height and z-chunk length it supports,
 * keeps the fastest as the context's options and returns the tile height
 * and z chunk. It never changes a value: the warp-specialised kernel
 * (LC2_OPTION_PIPELINE) and the resampling form (LC2_OPTION_PRESAMPLE) stay
 * as the caller set them. Contexts
 * without a tunable kernel (2D windows, mutual information, the generic
 * path) return their current settings. The reference takes fixed block sizes as
 * arguments (src/cu_LC2/cu_lc2_3d.cuh:36-41). */
int lc2_autotune(lc2_context* ctx, const float* matrices, int count, int* tile_rows, int* zchunk);

/* Per-kernel device timing with CUDA events on the context stream (off by
 * default). lc2_kernel_times synchronises, returns the summed milliseconds
 * and launch counts of the resampling, Sobel and moments kernels since the
 * last call (index 0, 1, 2), and resets them. */
int lc2_enable_kernel_timing(lc2_context* ctx, int on);
int lc2_kernel_times(lc2_context* ctx, double ms[3], long long counts[3]);

/* Transform builders. Replace Spatial3DMapper::AffineInit / RigidInit
 * (src/Interpolator/spatialMappers.cuh:585-850) and Spatial2DMapper::AffineInit
 * (:999-1033): x_m = L (x_v - C + shift) + C + T, L = Rz Ry Rx Sh S (3D),
 * L = R Sh S (2D). Angles in degrees; outputs row-major float matrices. */
int lc2_affine_3d(const float rotation[3], const float translation[3], const float scale[3],
                  const float shear[3], const float center[3], const float shift[3],
                  float out[16]);
int lc2_affine_2d(float rotation, const float translation[2], const float scale[2], float shear,
                  const float center[2], const float shift[2], float out[9]);

/* Inverse of a row-major affine 4x4 (bottom row 0 0 0 1). Replaces
 * InvertS4X4Matrix (src/Utilities/my_cuda_helper.cu:395-523) and
 * Spatial3DMapper::GetMyselfInversed (spatialMappers.cuh:315-433). Returns
 * LC2_ERR_SINGULAR when the determinant is 0. */
int lc2_invert_affine_3d(const float in[16], float out[16]);

/* ---- Optimizers (NLopt's role in the reference) ----
 * Derivative-free, bound-constrained minimisation whose objective receives a
 * batch of points per call (count x dim, row-major) and writes count values;
 * a non-zero return aborts with that status. Replaces the NLopt calls of
 * Optimizers{2D,3D,2DTo3D}::Optimize (src/Optimizers/optimizers.cu:298-302,
 * 385-390, 854-863, 937-946, 1473-1477, 1548-1553): LC2_OPT_DIRECT_L for
 * GN_ORIG_DIRECT_L, LC2_OPT_BOBYQA for LN_BOBYQA (Powell's 2009 method: 2n+1
 * interpolation points, least-Frobenius-norm model updates, bounded
 * trust-region and geometry steps; one evaluation per iteration after the
 * first 2n+1, which come as one batch), LC2_OPT_NELDER_MEAD for
 * LN_NELDERMEAD. LC2_OPT_QUAD_TR (no NLopt counterpart) is a batched
 * separable quadratic-model trust region that evaluates a 2n+1-point stencil
 * per step. xtol_rel (rho_end of BOBYQA) and initial_step (its rho_beg) are
 * measured in units of (upper - lower) per entry. */
typedef int (*lc2_batch_objective)(void* user, int count, int dim, const double* x, double* f);
enum { LC2_OPT_DIRECT_L = 1, LC2_OPT_BOBYQA = 2, LC2_OPT_NELDER_MEAD = 3, LC2_OPT_QUAD_TR = 4 };
typedef struct {
    int algorithm;        /* LC2_OPT_* */
    int dim;
    const double* lower;  /* dim entries */
    const double* upper;
    double xtol_rel;      /* stop when steps fall below xtol_rel * (upper - lower) */
    int maxeval;          /* 0 = no limit */
    double initial_step;  /* fraction of (upper - lower); 0 = 0.1 */
} lc2_opt_problem;
typedef struct {
    int evaluations;
    int batches;          /* objective calls (one batched launch each) */
} lc2_opt_report;
/* Minimises f from x (clamped to the bounds); x receives the best point. */
int lc2_minimize(const lc2_opt_problem* problem, lc2_batch_objective f, void* user, double* x,
                 double* fmin, lc2_opt_report* report);

/* Registration driver: the DIRECT stage on the entries of direct_entries,
 * then up to 8 local rounds on their entries, minimising -log(LC2) with
 * every optimizer step evaluated as one batched launch on `ctx`. Mirrors
 * Optimizers{2D,3D}::Optimize (src/Optimizers/optimizers.cu:183-410,
 * 734-970). Parameters follow the reference's order: 2D TX TY R ScaleX
 * ScaleY Shear (6); 3D and 2D-to-3D TX TY TZ RX RY RZ ScaleX..Z ShearX..Z
 * (12). Bounds are absolute (the reference adds its translation and
 * rotation bounds to InitialValues, optimizers.cu:46-57, before this). */
enum { LC2_ENTRY_TRANSLATION = 1, LC2_ENTRY_ROTATION = 2, LC2_ENTRY_SCALE = 4,
       LC2_ENTRY_SHEAR = 8 };
typedef struct {
    int mode;              /* must match the context */
    double initial[12];
    double lower[12];
    double upper[12];
    float center[3];       /* rotation centre: the fixed image's centre */
    float shift[3];        /* moving centre - virtual centre when centred, else 0 */
    int direct_entries;    /* LC2_ENTRY_* mask; 0 = no DIRECT stage */
    int direct_maxeval;
    int rounds;            /* local rounds (<= 8) */
    int round_entries[8];  /* LC2_ENTRY_* mask per round; 0 = round disabled */
    double round_xtol[8];  /* the round's AbsTol */
    int round_maxeval;     /* per round; 0 = no limit */
    int local_algorithm;   /* LC2_OPT_BOBYQA (default), LC2_OPT_NELDER_MEAD or
                            * LC2_OPT_QUAD_TR */
    /* When lc2_register gets no context: LC2 of `count` matrices (row-major
     * 3x3 or 4x4 as doubles, dim = 9 or 16) from this callback instead, e.g.
     * a reference implementation for comparisons. */
    lc2_batch_objective lc2_of_matrices;
    void* user;
    /* Optional: called after every batch with the stage (0 = DIRECT, r + 1 =
     * local round r, rounds + 1 = the final evaluation at the optimum), the
     * `count` parameter vectors (reference order, 6 or 12 entries each) and
     * their LC2 values, e.g. to write RegistrationInfo.log
     * (src/Optimizers/optimizers.cu:709-720). Every evaluation counted in
     * lc2_registration_result.evaluations is reported exactly once. */
    void (*observer)(void* user, int stage, int count, int nparams, const double* params,
                     const double* lc2);
    void* observer_user;
    /* 1: the similarity is maximised as it is (normalised mutual information,
     * src/Optimizers/optimizers.cu:722-724, 855-860); 0: -log(LC2) is
     * minimised. Set automatically for a context with patch_size 0. */
    int maximize;
} lc2_registration;
typedef struct {
    double params[12];     /* optimum, reference order */
    double lc2;            /* LC2 at the optimum */
    int evaluations;
    int launches;          /* batched objective launches */
} lc2_registration_result;
int lc2_register(lc2_context* ctx, const lc2_registration* reg, lc2_registration_result* out);
/* the similarity of one parameter vector as lc2_register sees it */
int lc2_params_to_matrix(int mode, const double* params, const float center[3],
                         const float shift[3], float* matrix);

/* ---- Serving ----
 * A request loop for whole registrations (the reference registers one
 * request per process, src/mainRegistrationTool/main.cu:728-801). Requests
 * are admitted in arrival order while their device memory fits the budget
 * and fewer than max_active are running; each admitted request runs on its
 * own worker thread with its own context and CUDA stream, so the kernels of
 * concurrent requests overlap on the GPU, and a request's images, weighting
 * factors and optimizer state stay resident until it completes. The
 * optimizer steps of concurrent 2D and 2D-to-3D requests are evaluated
 * together in merged launches (merge_window_us). Results are identical to
 * the same request registered alone (lc2_register). */
typedef struct lc2_server lc2_server;
typedef struct {
    size_t hbm_budget_bytes; /* device bytes admitted requests may hold; 0 = 80% of free memory */
    int max_active;          /* registrations in flight (worker threads); 0 = 8 */
    int device;              /* CUDA device of every request */
    int merge_window_us;     /* cross-request batching of 2D and 2D-to-3D registrations
                              * (HighResolutionModality Moving, PatchSize >= 1): the
                              * optimizer steps of concurrent requests of one mode, patch
                              * size and storage type are evaluated in one lc2_merger
                              * launch; a step waits at most this long for the other
                              * running requests' steps. 0 = 200 us, < 0 = off (each
                              * request launches on its own stream). */
} lc2_server_config;
typedef struct {
    lc2_config config;       /* images, patch, storage (config.device is replaced by the server's) */
    const float* fixed;      /* host images, copied by lc2_server_submit */
    const float* moving;
    /* optimizer settings; with registration.lc2_of_matrices set the request
     * runs that host objective and touches no GPU */
    lc2_registration registration;
} lc2_request;
typedef struct {
    int status;                      /* lc2_status of the registration */
    char message[160];               /* lc2_last_error() of a failed request */
    lc2_registration_result result;
    double queue_ms, run_ms, total_ms; /* submit->admission, admission->done, submit->done */
    size_t device_bytes;             /* budget the request held while running */
    long long admission;             /* admission order 0, 1, ... */
} lc2_request_result;
typedef struct {
    long long submitted, completed, failed;
    int queued, active, peak_active;
    size_t budget_bytes, bytes_in_use, peak_bytes;
    double p50_ms, p95_ms, p99_ms, mean_ms; /* total latency of completed requests */
    double elapsed_s;                /* since creation or the last reset */
    long long merged_launches;       /* merged launches since creation */
    long long merged_steps;          /* optimizer steps they carried (one per request each) */
} lc2_server_stats;

/* A 2D-to-3D stack request: one moving volume, `frames` ultrasound frames
 * (geometries frame_geoms[i], images frame_images[i], one shared virtual
 * spacing) and one registration per frame (mode LC2_MODE_2DTO3D), run as
 * lc2_stack_register. Host buffers are copied by the submit call. */
typedef struct {
    lc2_geometry moving;
    const float* moving_image;
    int patch_size;
    int storage;
    int frames;
    const lc2_geometry* frame_geoms;
    const float* const* frame_images;
    float virtual_spacing[3];
    const lc2_registration* registrations;
} lc2_stack_request;

/* Device bytes a context of this configuration holds (*held) and at most
 * while lc2_set_images runs (*peak, may be NULL). No device work. */
int lc2_context_bytes(const lc2_config* cfg, size_t* held, size_t* peak);
int lc2_server_create(const lc2_server_config* cfg, lc2_server** out);
/* Queues a request; *ticket identifies it. LC2_ERR_OUT_OF_MEMORY when the
 * request alone exceeds the budget. */
int lc2_server_submit(lc2_server* s, const lc2_request* req, long long* ticket);
/* Queues a stack request; polled with lc2_server_poll_stack. */
int lc2_server_submit_stack(lc2_server* s, const lc2_stack_request* req, long long* ticket);
/* As lc2_server_poll for a stack request: out receives one result per frame
 * (`frames` entries), each with the request's queue / run / total times. */
int lc2_server_poll_stack(lc2_server* s, long long ticket, int wait_ms, lc2_request_result* out,
                          int frames);
/* Waits up to wait_ms (-1 = no limit) for the request; LC2_ERR_NOT_READY
 * while it is queued or running. A completed result is returned once. */
int lc2_server_poll(lc2_server* s, long long ticket, int wait_ms, lc2_request_result* out);
/* Waits up to wait_ms (-1 = no limit) until nothing is queued or running. */
int lc2_server_drain(lc2_server* s, int wait_ms);
int lc2_server_get_stats(lc2_server* s, lc2_server_stats* out);
int lc2_server_reset_stats(lc2_server* s);
/* Finishes running requests, drops queued ones, joins the workers. */
int lc2_server_destroy(lc2_server* s);

/* ---- 2D-to-3D frame stacks ----
 * One MR/CT volume against many ultrasound frames of their own sizes and
 * geometries, with any number of candidate poses per frame, evaluated in one
 * persistent launch (replayed from a CUDA graph when the frame layout of a
 * call repeats). Each frame behaves exactly as an LC2_MODE_2DTO3D context
 * with HighResolutionModality: Moving (Interpolator2DTo3D,
 * src/Interpolator/interpolator.cu:1538-1775; LC2_2D_class on the frame,
 * src/cu_LC2/cu_lc2_2d.cu:515-653) that shares the stack's volume: a stack
 * evaluation returns the same value, bit for bit, as lc2_evaluate on a
 * standalone context of that frame. The reference evaluates one frame and
 * one pose per call. */
typedef struct lc2_stack lc2_stack;

/* Creates an empty stack for a moving volume of geometry `moving`, patch
 * radius `patch_size` (1..12), storage type (lc2_storage) on `device`. */
int lc2_stack_create(const lc2_geometry* moving, int patch_size, int storage, int device,
                     lc2_stack** out);
/* Releases the stack, its frames and their device memory. */
int lc2_stack_destroy(lc2_stack* s);
/* Uploads the moving volume (host float32). Once per stack, before frames. */
int lc2_stack_set_moving(lc2_stack* s, const float* moving);
/* Adds a frame: its geometry (dim[2] = 1), virtual spacing and ultrasound
 * image (host float32); returns its id (0, 1, ...) in *frame_id. */
int lc2_stack_add_frame(lc2_stack* s, const lc2_geometry* frame, const float virtual_spacing[3],
                        const float* ultrasound, int* frame_id);
/* Number of frames. */
int lc2_stack_frames(const lc2_stack* s);
/* The frame's own context (owned by the stack; do not destroy or call
 * lc2_set_images on it), e.g. for lc2_evaluate or lc2_register on one frame. */
int lc2_stack_frame_context(lc2_stack* s, int frame_id, lc2_context** ctx);
/* `count` evaluations: frame_ids[k] with the 4x4 virtual->moving matrix
 * matrices[16 k ..]; lc2[k] receives the LC2 value. Frames may repeat and
 * come in any order. */
int lc2_stack_evaluate(lc2_stack* s, int count, const int* frame_ids, const float* matrices,
                       double* lc2);
/* CUDA-graph replay of repeated layouts: on (1, default) or off (0). */
int lc2_stack_set_graphs(lc2_stack* s, int on);
/* LC2_OPTION_GRAPHS and LC2_OPTION_STREAM_PRIORITY for the stack's own
 * stream (as lc2_set_option), and LC2_OPTION_STACK_BATCHING for
 * lc2_stack_register: 1 (default) evaluates every round of the frames'
 * optimizer steps as one stack launch (throughput), 0 runs the frames'
 * registrations independently and concurrently on their own contexts and
 * streams (latency; frame ids must then be distinct). Same results. */
enum { LC2_OPTION_STACK_BATCHING = 6 };
int lc2_stack_set_option(lc2_stack* s, int option, int value);
int lc2_stack_get_option(const lc2_stack* s, int option, int* value);
/* Registers n frames at once (Optimizers2DTo3D per frame,
 * src/Optimizers/optimizers.cu:1195-1640): regs[i] (mode LC2_MODE_2DTO3D)
 * on frame frame_ids[i], each on its own host thread, with every round of
 * their optimizer steps evaluated as one stack launch. results[i] equals
 * lc2_register on that frame's context alone. statuses (may be NULL): per
 * registration lc2_status; *launches (may be NULL): stack evaluations issued.
 * Returns the first failure, else LC2_OK. */
int lc2_stack_register(lc2_stack* s, int n, const int* frame_ids, const lc2_registration* regs,
                       lc2_registration_result* results, int* statuses, long long* launches);
/* Kernel launches and graph launches issued by the stack since creation. */
long long lc2_stack_launch_count(const lc2_stack* s);
long long lc2_stack_graph_launches(const lc2_stack* s);

/* ---- Cross-context batching ----
 * Evaluations of several contexts -- e.g. the optimizer steps of concurrent
 * registrations -- in one launch of the work-list kernel that 2D-to-3D stacks
 * use (one segment per context, each with its own images, grid and
 * fixed-point scales). The reference evaluates one transform of one
 * registration per call (src/Optimizers/optimizers.cu:130-181); this has no
 * counterpart there. Contexts must be 2D or 2D-to-3D, HighResolutionModality
 * Moving, PatchSize >= 1, with images set, and share the mode, patch size,
 * storage type and the merger's device. Values equal lc2_evaluate_batch on
 * each context bit for bit. A merger is used by one host thread at a time. */
typedef struct lc2_merger lc2_merger;
int lc2_merger_create(int device, lc2_merger** out);
int lc2_merger_destroy(lc2_merger* m);
/* counts[i] transforms of ctxs[i]; matrices and lc2_out hold all of them in
 * context order (3x3 in 2D mode, 4x4 in 2D-to-3D mode). */
int lc2_merger_evaluate(lc2_merger* m, int n, lc2_context* const* ctxs, const int* counts,
                        const float* matrices, double* lc2_out);
/* Kernel launches issued by the merger since creation. */
long long lc2_merger_launch_count(const lc2_merger* m);

/* Evaluation for callers that cannot allocate device memory: a host
 * application whose allocator or memory pool owns the device heap, a
 * real-time loop that must not allocate after start-up, a plug-in handed
 * device buffers and nothing else. No counterpart in the reference.
 *
 * Inputs and output are the caller's device buffers: d_ultrasound is the
 * ultrasound already on the virtual grid `virt` (float32, x fastest; the
 * ultrasound is the fixed image, i.e. HighResolutionModality: Moving),
 * d_moving the moving image with geometry `moving`, matrix the host-side
 * virtual->moving matrix (3x3 in 2D mode, 4x4 otherwise) and d_lc2 one
 * device double that receives the LC2 value. All work is enqueued on
 * `stream` (a cudaStream_t, NULL = default stream); the call returns after
 * reading back the input maxima, with the result still pending on `stream`.
 *
 * No memory is allocated: the resampled image, its Sobel magnitude and the
 * sums live in one static device array of 256 B + 8 B per voxel for at most
 * LC2_NOALLOC_MAX_VOXELS virtual voxels (8 MiB), which every GPU that loads
 * the library holds until the process exits; larger grids are rejected with
 * LC2_ERR_UNSUPPORTED, as are moving images of more than 2^31 - 1 voxels.
 * The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress, with the device current, in the device's primary
 * context; a cudaDeviceReset invalidates it for the rest of the process).
 * Every call blocks the host on a read-back of the input maxima, so none can
 * be recorded into a CUDA graph: on a capturing stream the call returns
 * LC2_ERR_UNSUPPORTED before enqueuing anything. Every call shares the
 * array: calls that overlap on the GPU (other streams, other host threads on
 * the same device) race and must be serialised by the caller. */
#define LC2_NOALLOC_MAX_VOXELS (1 << 20)
int lc2_evaluate_noalloc(int mode, const lc2_geometry* virt, const lc2_geometry* moving,
                         int patch_size, const float* d_ultrasound, const float* d_moving,
                         const float* matrix, double* d_lc2, void* stream);

/* Test hooks for the failure paths (no counterpart in the reference, which
 * checks no allocation). lc2_debug_fail_allocation(k): the k-th device or
 * pinned-host allocation the library makes from now on (any thread) fails
 * as an out-of-memory would, without calling CUDA; k = 0 disarms it.
 * lc2_debug_device_bytes: device bytes and allocations the library holds
 * now, to check that a failed call released what it had taken. */
int lc2_debug_fail_allocation(long long k);
int lc2_debug_device_bytes(size_t* live_bytes, long long* live_allocations);

/* Message of the last failure on the calling thread ("" if none). */
const char* lc2_last_error(void);

/* Library version string. */
const char* lc2_version(void);

#ifdef __cplusplus
}
#endif
#endif
