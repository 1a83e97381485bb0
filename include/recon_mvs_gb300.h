/*
 * recon_mvs_gb300.h -- C ABI of the GB300 PatchMatch multi-view-stereo
 * engine (librecon_mvs_gb300.so).
 *
 * A drop-in for the MVS path of kai3934908500/recon-scanner:
 *   core/include/recon/mvs.h:133-214 (SelectSourceViews, ComputeNcc,
 *   PatchMatchStereo, RefineSubpixel, FuseDepthMaps) and the conventions of
 *   core/include/recon/recon_c_api.h (POD structs, recon_status returns, no
 *   exception crosses the boundary, core-allocated buffers freed by the
 *   library).  Every entry point below names the reference interface it
 *   replaces.
 *
 * Memory: unless stated otherwise every pointer is HOST memory owned by the
 * caller and only read/written during the call.  Images are tightly packed
 * 8-bit grayscale (stride = width), as in the reference.
 *
 * Threading: one context per host thread; the stateless entry points use a
 * per-thread default context on the options' device.
 *
 * When recon_c_api.h is used as well, include it first: the shared types
 * (recon_camera_intrinsics, recon_pose, recon_status) are then taken from it.
 */
#ifndef RECON_MVS_GB300_H_
#define RECON_MVS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RECON_MVS_GB300_ABI_VERSION 1

/* recon_c_api.h:31-37 */
#ifndef RECON_API
#if defined(__GNUC__) || defined(__clang__)
#define RECON_API __attribute__((visibility("default")))
#else
#define RECON_API
#endif
#endif

#ifndef RECON_RECON_C_API_H_
/* Same layout as recon_camera_intrinsics (recon_c_api.h:44-56). */
typedef struct recon_camera_intrinsics {
  double fx, fy, cx, cy;
  double k1, k2, k3, p1, p2;
  double width, height;
} recon_camera_intrinsics;

/* Same layout as recon_pose (recon_c_api.h:59-63): world -> camera,
 * r row-major, t in metres. */
typedef struct recon_pose {
  double r[9];
  double t[3];
  double timestamp_ns;
} recon_pose;

/* The subset of recon_status (recon_c_api.h:135-207) this engine returns,
 * with the reference's numeric values. */
typedef enum recon_status {
  RECON_OK = 0,
  RECON_ERR_INVALID_ARGUMENT = 1,
  RECON_ERR_OUT_OF_MEMORY = 2,
  RECON_ERR_NOT_IMPLEMENTED = 3,
  RECON_ERR_INTERNAL = 4,
  RECON_ERR_CANCELLED = 5,
  RECON_ERR_MVS_NO_DEPTH = 500,
  RECON_ERR_MVS_FILTER_EXHAUSTED = 501,
  RECON_ERR_MVS_GPU_FAILURE = 502
} recon_status;
#endif

/* recon::MvsConfig (core/include/recon/mvs.h:24-67), field for field and in
 * order; bool fields are int32.  recon_mvs_config_default() gives the
 * reference defaults. */
typedef struct recon_mvs_config {
  int32_t num_views;
  int32_t ref_view_index;
  double ideal_angle_min_deg;
  double ideal_angle_max_deg;
  double max_view_scale_mismatch;
  double view_angle_weight;
  double view_texture_weight;
  double view_spread_weight;
  double view_scale_weight;
  double reference_depth_m;
  int32_t patch_size;
  int32_t iterations;
  int32_t random_search_count;
  double random_search_radius_ratio;
  double restart_ratio;
  int32_t propagation_directions;
  int32_t propagation_enabled;
  int32_t num_threads;
  double photo_threshold;
  double depth_regularization;
  double geo_consistency_threshold;
  double weak_texture_variance;
  int32_t subpixel_iterations;
  int32_t subpixel_fit_points;
  double subpixel_window_ratio;
  double min_depth_m;
  double max_depth_m;
  int32_t min_view_consistency;
  double fusion_voxel_size_m;
} recon_mvs_config;

/* Search model. */
typedef enum recon_mvs_mode {
  /* The reference algorithm (patchmatch_stereo.cpp:422-764): fronto-parallel
   * inverse-depth hypotheses, translated NCC windows, mean NCC over valid
   * views, its Jacobi direction sweeps and row-block xorshift draws.  Depth
   * maps match the reference's up to FP32-vs-FP64 cost rounding; results
   * depend on num_threads exactly as the reference's do. */
  RECON_MVS_MODE_COMPAT = 0,
  /* The GB300 engine: plane hypotheses (inverse depth + normal), per-sample
   * homography windows, mean of the best_k view costs, red-black
   * checkerboard propagation with adaptive neighbour selection and random
   * perturbation.  Requires undistorted (pinhole) images. */
  RECON_MVS_MODE_PLANE = 1
} recon_mvs_mode;

typedef enum recon_mvs_storage {
  RECON_MVS_STORAGE_FP32 = 0, /* source images as FP32 textures */
  RECON_MVS_STORAGE_FP16 = 1, /* FP16 textures: exact for 8-bit input */
  RECON_MVS_STORAGE_BF16 = 2, /* BF16 values (8-bit mantissa; an ablation of FP16) in 16-bit textures,
                                 read by 2x2 gather and widened exactly; plane mode, interp = 0 only */
  RECON_MVS_STORAGE_U8 = 3    /* 8-bit textures read as I / 255 (NCC does not see the scale): the
                                 bandwidth floor, exact for 8-bit input; resampled (undistorted)
                                 intensities are rounded to 8 bits; plane mode only */
} recon_mvs_storage;

typedef struct recon_mvs_options {
  int32_t mode;       /* recon_mvs_mode */
  int32_t storage;    /* recon_mvs_storage */
  int32_t best_k;     /* plane mode: views averaged per hypothesis, <= 8; 0 = all valid */
  int32_t refine;     /* plane mode refinement after the sweeps: 0 none; 1 golden-section search of
                         the inverse depth (the reference's schedule, subpixel_iterations steps);
                         2 one Gauss-Newton step on depth and normal driven by the adjoint
                         (recon_mvs_job_adjoint), kept only if the cost falls */
  uint64_t seed;      /* plane mode random stream */
  int32_t device;     /* CUDA device ordinal */
  int32_t sampling;   /* plane mode: 0 = pixel-centre windows; 1 = the reference's convention
                         (window samples at x + 0.5 + dx read with index == coordinate, i.e. a
                         2x2-box reference window and unshifted source coordinates) */
  int32_t prefilter;  /* 1 = smooth every image with a 3x3 binomial ([1 2 1]/4 each way) when it is
                         staged: a shift-free low-pass that removes aliasing noise symmetrically */
  int32_t interp;     /* plane mode: 0 = exact FP32 bilinear interpolation (2x2 texel gather);
                         1 = the texture unit's bilinear filter (8-bit fixed-point weights: ~2x
                         fewer instructions per sample, costs within ~1e-3 of the exact ones) */
  int32_t tile_rows;  /* plane mode: rows per work tile of the persistent sweep (2, 4 or 8);
                         0 = chosen by the autotuner (timed once per batch shape, cached) */
  int32_t per_view;   /* plane mode: 0 = the jobs of one run form one batch -- one launch per
                         stage over all of them, captured once as a CUDA graph and replayed;
                         1 = the same kernels launched once per view, no graph */
  int32_t exhaustive; /* plane mode: 1 = evaluate every candidate on every source window; 0 = skip
                         a propagation candidate equal to the one just rejected, and the remaining
                         windows of a candidate once its best-k bound shows it cannot be taken (the
                         maps are the same; a switch for checks and timing) */
  int32_t coarse_iterations; /* plane mode: 0 = off; n > 0 (and n < the configured iterations) = the
                                first n iterations run on a half-resolution pyramid level (2x2 means of
                                the staged images, focal lengths and principal point halved), and the
                                full-resolution search starts from the planes they found: coarse-to-fine
                                initialisation, the configured iteration count in total */
  int32_t window_staging;    /* plane mode sweep, exact interpolation with FP32 or FP16 storage, 7x7 or
                                11x11 windows: 0 = the autotuner picks the window schedule; 1 = every
                                source sample read by the texture unit (2x2 gather); 2 = staged: per
                                candidate and source view each warp copies the source box its windows
                                cover (up to 40 x 24 texel pairs) into shared memory by TMA and
                                samples it there, windows whose box does not fit read the texture.  The
                                maps are the same bit for bit in every schedule */
  int32_t exploration_iterations; /* plane mode exploration schedule: 0 = every sweep evaluates the two
                                exploration candidates (a uniformly random plane; the current depth on a
                                fronto-parallel plane); n > 0 = only iterations 0 .. n-1 (counted over the
                                whole schedule, coarse-to-fine levels included) do, later sweeps keep
                                propagation and the local perturbations.  The random draws are made
                                either way, so iterations before n are unchanged */
} recon_mvs_options;

/* Inputs of one reference view: the PatchMatchStereo argument list
 * (mvs.h:164-177) with its index contract (mvs.h:151-161): src_gray /
 * src_w / src_h use the relative index k; poses the global index
 * source_indices[k]; src_intrinsics are global when num_src_intrinsics ==
 * num_src_poses, else relative when == num_src. */
typedef struct recon_mvs_views {
  const uint8_t* ref_gray;
  int32_t ref_w, ref_h;
  int32_t num_src;
  const uint8_t* const* src_gray;
  const int32_t* src_w;
  const int32_t* src_h;
  const recon_pose* ref_pose;
  const recon_pose* src_poses;
  int32_t num_src_poses;
  const recon_camera_intrinsics* ref_intr;
  const recon_camera_intrinsics* src_intrinsics;
  int32_t num_src_intrinsics;
  const int32_t* source_indices;
} recon_mvs_views;

/* recon::DepthMap (mvs.h:85-109), caller-allocated width*height arrays.
 * depth NaN = invalid.  normal (3 floats per pixel, reference camera
 * frame) and cost are optional outputs (NULL = not wanted). */
typedef struct recon_mvs_depth_map {
  int32_t width, height;
  float* depth;
  uint8_t* support_count;
  float* confidence;
  float* normal;
  float* cost;
} recon_mvs_depth_map;

/* recon::NccResult (mvs.h:70-75). */
typedef struct recon_mvs_ncc_result {
  int32_t valid;
  double ncc;
  int32_t weak_texture;
  int32_t valid_samples;
} recon_mvs_ncc_result;

/* recon::PointCloud (mvs.h:112-125), library-allocated; release with
 * recon_mvs_point_cloud_free.  keys / counts are the voxel key of each
 * point and the number of pixels fused into it. */
typedef struct recon_mvs_point_cloud {
  int64_t count;
  double* positions;
  double* normals;
  float* colors;
  float* confidences;
  int64_t* keys;
  uint32_t* counts;
} recon_mvs_point_cloud;

typedef struct recon_mvs_stats {
  uint64_t hypotheses_evaluated; /* plane sweeps: hypotheses whose windows were evaluated */
  double last_run_ms;            /* device time of the last PatchMatch run (CUDA events) */
  double last_sweep_ms;          /* device time of its sweeps only */
  int32_t last_sweep_launches;
  int32_t tile_rows;             /* sweep tile rows of the last plane run */
  int32_t ctas_per_sm;           /* its persistent blocks per SM */
  int32_t graph_launches;        /* CUDA-graph replays so far */
  int32_t tune_trials;           /* autotuner searches run by this context */
  int32_t window_staging;        /* the sweep's window schedule in the last plane run: 1 = staged boxes */
  uint64_t windows_evaluated;    /* plane sweeps: source windows sampled (a hypothesis samples up to one
                                    per source; views that cannot change its fate are skipped) */
  uint64_t windows_staged;       /* of them, windows read from a staged shared-memory box */
} recon_mvs_stats;

/* ---- version and configuration ---------------------------------------- */

/* recon_abi_version (recon_c_api.h:430) */
RECON_API uint32_t recon_mvs_abi_version(void);
/* MvsConfig{} defaults (mvs.h:24-67) */
RECON_API void recon_mvs_config_default(recon_mvs_config* cfg);
RECON_API void recon_mvs_options_default(recon_mvs_options* opts);
/* recon_set_param (c_api.cpp:158-180) + ParamStore::Set clamping
 * (params.cpp:133-157) for the 15 mvs_* keys (params.h:162-177), mapped
 * onto MvsConfig as Orchestrator::StageMvs does (orchestrator.cpp:952-970).
 * Unknown keys: RECON_ERR_INVALID_ARGUMENT. */
RECON_API recon_status recon_mvs_config_set_param(recon_mvs_config* cfg, const char* key, int32_t value_int,
                                                  double value_double);
/* recon_apply_preset (recon_c_api.h:442): 0 fast, 1 standard, 2 high. */
RECON_API recon_status recon_mvs_config_apply_preset(recon_mvs_config* cfg, int32_t preset);

/* ---- the MVS functions --------------------------------------------------- */

/* recon::SelectSourceViews (mvs.h:133-136; patchmatch_stereo.cpp:133-211).
 * Host-side geometry; writes up to `capacity` global indices. */
RECON_API recon_status recon_mvs_select_source_views(const recon_pose* ref_pose, const recon_pose* poses,
                                                     int32_t num_poses, const recon_camera_intrinsics* intr,
                                                     const recon_mvs_config* cfg, int32_t* out_indices,
                                                     int32_t capacity, int32_t* out_count);

/* recon::ComputeNcc (mvs.h:144-146; patchmatch_stereo.cpp:214-274) for n
 * windows (coords: n x {ref_u, ref_v, src_u, src_v}); FP64 on the GPU,
 * bit-identical to the reference. */
RECON_API recon_status recon_mvs_compute_ncc(const uint8_t* ref, int32_t ref_w, int32_t ref_h, const uint8_t* src,
                                             int32_t src_w, int32_t src_h, const double* coords, int32_t n,
                                             int32_t patch_size, recon_mvs_ncc_result* out);

/* Cost of n given hypotheses at integer pixels (px, py): the
 * EvaluateCandidate of patchmatch_stereo.cpp:344-418 in COMPAT mode
 * (inv_depth only), the plane cost in PLANE mode (inv_depth + normals,
 * 3 floats each).  out_view_cost (n x num_src, optional) holds 1 - NCC per
 * view, 1e30 for invalid views. */
RECON_API recon_status recon_mvs_evaluate(const recon_mvs_views* views, const recon_mvs_config* cfg,
                                          const recon_mvs_options* opts, int32_t n, const int32_t* px,
                                          const int32_t* py, const double* inv_depth, const float* normals,
                                          float* out_cost, int32_t* out_support, float* out_view_cost);

/* recon::PatchMatchStereo (mvs.h:164-177).  seed_points: num_seeds x
 * {u, v, depth_m} or NULL.  Contract violations (mvs.h:151-161) return
 * RECON_ERR_INVALID_ARGUMENT and leave `out` untouched, where the reference
 * returns 0; a degenerate baseline or depth range returns RECON_OK with
 * *out_filled = 0 and an all-invalid map, as the reference does. */
RECON_API recon_status recon_mvs_patchmatch(const recon_mvs_views* views, const recon_mvs_config* cfg,
                                            const recon_mvs_options* opts, const double* seed_points,
                                            int32_t num_seeds, recon_mvs_depth_map* out, uint32_t* out_filled);

/* recon::RefineSubpixel (mvs.h:185-196; patchmatch_stereo.cpp:770-979):
 * the reference's 5-point parabola + golden-section refinement of every
 * valid pixel, in place. */
RECON_API recon_status recon_mvs_refine_subpixel(const recon_mvs_views* views, const recon_mvs_config* cfg,
                                                 const recon_mvs_options* opts, recon_mvs_depth_map* depth,
                                                 uint32_t* out_refined);

/* Multi-view geometric consistency of map `ref_index` against the others
 * (spec: shaders/vulkan/recon_mvs_consistency.comp:94-140 with the strict
 * transform of shaders/common/gpu_algo.h:537-538, plus a reprojection
 * bound).  out_count: consistent maps per pixel; out_keep: count >=
 * min_views (both width*height of the reference map). */
RECON_API recon_status recon_mvs_geometric_consistency(const recon_mvs_depth_map* maps, const recon_pose* poses,
                                                       const recon_camera_intrinsics* intr, int32_t num_maps,
                                                       int32_t ref_index, float rel_depth_max, float reproj_px_max,
                                                       int32_t min_views, uint8_t* out_count, uint8_t* out_keep);

/* recon::FuseDepthMaps (mvs.h:203-206; patchmatch_stereo.cpp:985-1089).
 * keep_masks (optional, one per map, may contain NULLs) drop pixels before
 * fusion (the geometric-consistency filter).  The cloud is bit-identical to
 * the reference's; points come in order of the first pixel of each voxel. */
RECON_API recon_status recon_mvs_fuse(const recon_mvs_depth_map* maps, const recon_pose* poses,
                                      const recon_camera_intrinsics* intr, int32_t num_maps,
                                      const recon_mvs_config* cfg, const uint8_t* const* keep_masks,
                                      recon_mvs_point_cloud* out);
/* recon_free_buffer (recon_c_api.h:435-436) for point clouds. */
RECON_API void recon_mvs_point_cloud_free(recon_mvs_point_cloud* cloud);

/* Undistortion remap of an 8-bit image to the pinhole camera with the same
 * fx, fy, cx, cy (inverse map through ApplyDistortion, camera.cpp:33-45);
 * out: width*height floats, 0 outside the source. */
RECON_API recon_status recon_mvs_undistort(const uint8_t* img, int32_t w, int32_t h,
                                           const recon_camera_intrinsics* intr, float* out);

/* ---- device-resident jobs (batching and measurement) --------------------- */

/* A context owns a CUDA stream, device workspaces and staged jobs. */
RECON_API recon_status recon_mvs_context_create(const recon_mvs_options* opts, void** out_ctx);
RECON_API void recon_mvs_context_destroy(void* ctx);
/* Upload and prepare one reference view (images to textures, camera
 * tables); the job keeps the device copies until released.  When
 * undistort != 0 the images are first remapped to the pinhole camera
 * (recon_mvs_undistort) on the device. */
RECON_API recon_status recon_mvs_job_stage(void* ctx, const recon_mvs_views* views, const recon_mvs_config* cfg,
                                           int32_t undistort, int32_t* out_job);
/* Shared staging for a capture: an image is uploaded once (optionally
 * undistorted on the device; its intrinsics then become pinhole) and any
 * number of jobs use it -- as the reference of one map and a source of
 * others -- through recon_mvs_job_stage_images.  Jobs keep the images they
 * use alive; recon_mvs_image_release only drops the context's handle.  No
 * counterpart in the reference (its StageMvs passes the same keyframe
 * buffers to every PatchMatchStereo call). */
RECON_API recon_status recon_mvs_image_stage(void* ctx, const uint8_t* gray, int32_t w, int32_t h,
                                             const recon_camera_intrinsics* intr, int32_t undistort,
                                             int32_t* out_image);
/* A BGRA8 camera frame (rows `stride` bytes apart) staged as its gray image:
 * the conversion of BgraToGray (orchestrator.cpp:53-67, (77 R + 150 G + 29 B)
 * >> 8) runs on the device after the upload, then as recon_mvs_image_stage. */
RECON_API recon_status recon_mvs_image_stage_bgra(void* ctx, const uint8_t* bgra, int32_t w, int32_t h,
                                                  int32_t stride, const recon_camera_intrinsics* intr,
                                                  int32_t undistort, int32_t* out_image);
RECON_API recon_status recon_mvs_image_release(void* ctx, int32_t image);
/* A job from staged images: the reference image, num_src source images and
 * their world -> camera poses (src_poses[k] belongs to src_images[k]). */
RECON_API recon_status recon_mvs_job_stage_images(void* ctx, int32_t ref_image, int32_t num_src,
                                                  const int32_t* src_images, const recon_pose* ref_pose,
                                                  const recon_pose* src_poses, const recon_mvs_config* cfg,
                                                  int32_t* out_job);
/* Run PatchMatch (+ refinement per options) on staged jobs, asynchronously
 * on the context's stream.  Plane-mode jobs of one call run as one batch
 * (options.per_view); running the same job list again replays the batch's
 * captured CUDA graph.  Results do not depend on the batching. */
RECON_API recon_status recon_mvs_job_run(void* ctx, int32_t job);
RECON_API recon_status recon_mvs_jobs_run(void* ctx, const int32_t* jobs, int32_t n);
/* ---- the differentiation form (plane-mode jobs) ---- */

/* Adjoint of the aggregated plane cost at n hypotheses of a staged job: at
 * integer pixels (px, py), the depth d of the plane on the pixel-centre ray
 * and its normal as spherical angles angles[2i] = theta, angles[2i+1] = phi
 * (n = (sin t cos p, sin t sin p, cos t), reference camera frame).  Outputs
 * per hypothesis: the cost (mean of the best_k view costs, 1e30 invalid),
 * the gradient d cost / d (d, theta, phi) (3), optionally the Gauss-Newton
 * matrix (6: upper triangle 00 01 02 11 12 22) and the gradient in every
 * source's pose (num_src x 6: rotation w then translation tau of the left
 * perturbation Y' = exp([w]x) Y + tau of source-camera points; zero for views
 * outside the best_k).  Exact bilinear reads of the staged textures; every
 * window is recomputed for the reverse pass, never stored.  No counterpart in
 * the reference (its MVS has no derivatives). */
RECON_API recon_status recon_mvs_job_adjoint(void* ctx, int32_t job, int32_t n, const int32_t* px, const int32_t* py,
                                             const double* depth, const double* angles, float* out_cost,
                                             float* out_grad, float* out_gn, float* out_pose_grad);
/* Pose recovery: Levenberg-Marquardt on every source pose of a staged job,
 * minimising each view's mean 1 - NCC over the given hypotheses (held fixed;
 * every valid view counts, independent of best_k).  The job's source
 * transforms are updated in place (later runs of the job use them).
 * out_src_poses (num_src, optional): the refined world -> camera poses;
 * out_cost (iterations + 1, optional): the summed per-view mean cost before
 * and after each iteration.  No counterpart in the reference. */
RECON_API recon_status recon_mvs_job_recover_poses(void* ctx, int32_t job, int32_t n, const int32_t* px,
                                                   const int32_t* py, const double* depth, const double* angles,
                                                   int32_t iterations, recon_pose* out_src_poses,
                                                   double* out_cost);
/* BgraToGray (orchestrator.cpp:53-67) on the device: w x h gray bytes,
 * bit-identical to the reference's integer formula. */
RECON_API recon_status recon_mvs_bgra_to_gray(const uint8_t* bgra, int32_t w, int32_t h, int32_t stride,
                                              uint8_t* out);

/* ---- the MVS stage over a capture (Orchestrator::StageMvs) ---- */

typedef int32_t (*recon_mvs_cancel_fn)(void* user);              /* nonzero: cancel */
typedef void (*recon_mvs_progress_fn)(void* user, double fraction); /* maps done / maps */
typedef struct recon_mvs_stage_params {
  int32_t undistort;              /* stage images with on-device undistortion (plane mode needs it
                                     for distorted cameras) */
  int32_t batch_size;             /* maps per batched run; 0 = every map in one batch */
  int32_t consistency_views;      /* 0 = fuse every map as StageMvs does; n > 0 = fuse only pixels
                                     consistent with >= n other maps */
  int32_t plane_normals;          /* plane mode: 1 = fused normals from the plane hypotheses; 0 = the
                                     reference's -ray direction (FuseDepthMaps, bit-identical) */
  float consistency_rel_depth;    /* |z_back - z| / z bound of the consistency test */
  float consistency_reproj_px;    /* reprojection bound of the consistency test, pixels */
  recon_mvs_cancel_fn cancel;     /* optional, checked before every batch */
  recon_mvs_progress_fn progress; /* optional, called after every batch */
  void* user;
} recon_mvs_stage_params;

/* Orchestrator::StageMvs (orchestrator.cpp:942-1071) on the batched engine:
 * keyframes with their gray images (NULL = none), world -> camera poses and
 * intrinsics; per keyframe the sources of SelectSourceViews (without itself
 * and image-less frames, at most num_views); PatchMatch (+ the context's
 * refinement; RefineSubpixel in COMPAT mode) in batches; maps with nothing
 * filled dropped; fusion of the rest on the device into out_cloud (freed
 * with recon_mvs_point_cloud_free).  RECON_ERR_MVS_NO_DEPTH: fewer than two
 * keyframes or no map; RECON_ERR_CANCELLED: the cancel callback said so. */
RECON_API recon_status recon_mvs_stage_run(void* ctx, const uint8_t* const* gray, const int32_t* width,
                                           const int32_t* height, const recon_pose* poses,
                                           const recon_camera_intrinsics* intr, int32_t num_keyframes,
                                           const recon_mvs_config* cfg, const recon_mvs_stage_params* params,
                                           recon_mvs_point_cloud* out_cloud, int32_t* out_maps);
/* A fused point cloud left in device memory for the stage that consumes it
 * on the GPU (UnifiedPointCloud and its Poisson input,
 * orchestrator.cpp:1054-1064 and :181-193), so the cloud does not round-trip
 * through host memory.  Every array is device memory on `device`, owned by the
 * library, valid until recon_mvs_device_cloud_free; one record per voxel, in
 * the order recon_mvs_stage_run returns them. */
typedef struct recon_mvs_device_cloud {
  int64_t count;
  double* positions;   /* count x 3 */
  double* normals;     /* count x 3, unit */
  float* colors;       /* count x 3, zero (FuseDepthMaps writes no colour) */
  float* confidences;  /* count */
  float* weights;      /* count: Poisson point weights max(0, confidence) (ToOrientedCloud) */
  int64_t* keys;       /* count: voxel keys */
  uint32_t* counts;    /* count: points fused into each voxel */
  double bounds_lo[3]; /* PointCloudBounds of the positions without padding (orchestrator.cpp:80-99); */
  double bounds_hi[3]; /* +1e30 / -1e30 for an empty cloud */
  int32_t device;      /* CUDA device ordinal of the arrays */
  void* impl;
} recon_mvs_device_cloud;

/* recon_mvs_stage_run with the fused cloud kept in device memory (plus its
 * Poisson weights and bounds, computed on the device).  No counterpart in the
 * reference, whose cloud is a host vector. */
RECON_API recon_status recon_mvs_stage_run_device(void* ctx, const uint8_t* const* gray, const int32_t* width,
                                                  const int32_t* height, const recon_pose* poses,
                                                  const recon_camera_intrinsics* intr, int32_t num_keyframes,
                                                  const recon_mvs_config* cfg, const recon_mvs_stage_params* params,
                                                  recon_mvs_device_cloud* out_cloud, int32_t* out_maps);
/* Copy a device cloud into a host cloud (recon_mvs_point_cloud_free);
 * synchronises.  `ctx` must be a context on the cloud's device. */
RECON_API recon_status recon_mvs_device_cloud_download(void* ctx, const recon_mvs_device_cloud* cloud,
                                                       recon_mvs_point_cloud* out);
RECON_API void recon_mvs_device_cloud_free(recon_mvs_device_cloud* cloud);
/* Copy a finished job's map to the host (synchronises). */
RECON_API recon_status recon_mvs_job_download(void* ctx, int32_t job, recon_mvs_depth_map* out,
                                              uint32_t* out_filled);
RECON_API recon_status recon_mvs_job_release(void* ctx, int32_t job);
/* Test hook for the failure path of the sweep's bounded tile waits: the
 * next plane-mode run of this context issues no reference-tile copy and
 * waits at most 4096 polls for each, so every wait runs out; the run's
 * download then returns RECON_ERR_MVS_GPU_FAILURE and the context stays
 * usable (the following run is normal).  No counterpart in the reference. */
RECON_API recon_status recon_mvs_test_inject_tma_timeout(void* ctx);
RECON_API recon_status recon_mvs_synchronize(void* ctx);
RECON_API recon_status recon_mvs_context_stats(void* ctx, recon_mvs_stats* out);
/* Geometric consistency for callers that cannot let a library allocate
 * device memory -- for example a capture or streaming loop that keeps every
 * buffer in its own pre-sized pool (a cudaMalloc would synchronise the
 * device and stall it), or a process whose GPU memory is rationed by its own
 * allocator.  No counterpart in the reference.
 *
 * Same test as recon_mvs_geometric_consistency, but every map's `depth`
 * and out_count / out_keep (width*height of the reference map) are DEVICE
 * pointers owned by the caller; poses and intrinsics are host memory.  The
 * work is queued on `stream` (a cudaStream_t; NULL = the default stream).
 * The descriptor table is uploaded from pageable host memory, so the call
 * may block until the work already queued on that stream has drained; it
 * does not wait for the consistency kernel itself.  Nothing is allocated: the
 * per-source descriptor table lives in a fixed array in the library's
 * device image, sized for at most 64 source maps (num_maps - 1 <= 64; more
 * is RECON_ERR_INVALID_ARGUMENT).  Every GPU that loads the library keeps
 * that array until the process exits.
 *
 * Every call looks up the array's device address in the current CUDA
 * context (the address belongs to the context, not to the device number);
 * the first call in a context also loads the library's device image there,
 * so make that first call before any stream capture.  All calls share the
 * array and it keeps the last call's contents; calls whose GPU work overlaps
 * race on it, so serialise them. */
RECON_API recon_status recon_mvs_geometric_consistency_noalloc(const recon_mvs_depth_map* maps,
                                                               const recon_pose* poses,
                                                               const recon_camera_intrinsics* intr, int32_t num_maps,
                                                               int32_t ref_index, float rel_depth_max,
                                                               float reproj_px_max, int32_t min_views,
                                                               uint8_t* out_count, uint8_t* out_keep, void* stream);

/* ---- TSDF fusion (the RGBD branch) ----------------------------------------
 * recon::TsdfVolume (core/include/recon/tsdf_fusion.h:42-98,
 * core/src/rgbd/tsdf_fusion.cpp) with its grid in device memory: the same
 * dense grid, the same per-pixel ray walk and running weighted mean, applied
 * in the reference's order, so grids and extracted points are bit-identical
 * to the reference's. */
/* TsdfConfig (tsdf_fusion.h:17-39), field for field. */
typedef struct recon_tsdf_config {
  double voxel_size_m, truncation_m, min_depth_m, max_depth_m;
  double fx, fy, cx, cy;
  double origin_x, origin_y, origin_z;
  double bbox_max_x, bbox_max_y, bbox_max_z;
  int32_t min_confidence;
} recon_tsdf_config;
RECON_API recon_status recon_tsdf_config_default(recon_tsdf_config* out);
/* TsdfVolume::TsdfVolume: a grid of FloorToIntScaled(extent / voxel) + 1
 * voxels per axis on `device` (tsdf 1, weight 0); at most 2^31 voxels. */
RECON_API recon_status recon_tsdf_create(const recon_tsdf_config* cfg, int32_t device, void** out_volume);
/* TsdfVolume::IntegrateDepthFrame (tsdf_fusion.h:54-57): host depth in
 * uint16 millimetres of axial depth, optional uint8 confidence,
 * world_to_camera 4 x 4 row-major; *out_integrated = the pixels fused.
 * Synchronises. */
RECON_API recon_status recon_tsdf_integrate(void* volume, const uint16_t* depth_mm, const uint8_t* confidence,
                                            int32_t width, int32_t height, const double* world_to_camera,
                                            float depth_uncertainty_m, uint32_t* out_integrated);
/* TsdfVolume::ExtractPoints (tsdf_fusion.h:60-62): zero-crossing voxels in
 * (iz, iy, ix) order -- positions, normals, confidences; keys = linear voxel
 * index, counts = 1, colours 0 (freed with recon_mvs_point_cloud_free). */
RECON_API recon_status recon_tsdf_extract_points(void* volume, recon_mvs_point_cloud* out);
/* TsdfVolume::dims (x, y, z) and MemoryUsageBytes (the device grid: 8 bytes a
 * voxel; the reference also counts 12 bytes of colour it never writes). */
RECON_API recon_status recon_tsdf_dims(void* volume, int32_t* out_dims);
RECON_API recon_status recon_tsdf_memory_usage(void* volume, uint64_t* out_bytes);
/* Copies of the grid (nx * ny * nz floats each, index (iz * ny + iy) * nx +
 * ix; either may be NULL).  No counterpart in the reference, whose grid is
 * private. */
RECON_API recon_status recon_tsdf_read_grid(void* volume, float* tsdf, float* weight);
RECON_API void recon_tsdf_destroy(void* volume);

/* Human-readable description of the last error on this thread. */
RECON_API const char* recon_mvs_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* RECON_MVS_GB300_H_ */
