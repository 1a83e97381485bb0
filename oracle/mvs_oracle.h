/*
 * mvs_oracle.h -- CPU restatement of the reference PatchMatch MVS path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine:
 * only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
 * its `--impl reference` arm) may load it.  The product never links it and
 * never falls back to it.
 *
 * Every function restates, in plain C, one function of the reference
 * (kai3934908500/recon-scanner) with the same double-precision arithmetic in
 * the same evaluation order, so that, compiled with -ffp-contract=off, it
 * reproduces the reference bit for bit.  The pin is
 * tests/test_oracle_golden.py: golden vectors produced by the reference's own
 * sources (oracle/ref_wrapper.cpp, built by oracle/Makefile) are compared
 * with this restatement bit-exactly.
 *
 * Functions without a reference counterpart (the plane-induced homography
 * cost, the geometric-consistency test, the undistortion remap) are FP64
 * restatements of the formulas the GPU engine implements; their headers say
 * so.
 */
#ifndef RECON_MVS_ORACLE_H_
#define RECON_MVS_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as recon_camera_intrinsics (core/include/recon/recon_c_api.h:44-56). */
typedef struct orc_intrinsics {
  double fx, fy, cx, cy;
  double k1, k2, k3, p1, p2;
  double width, height;
} orc_intrinsics;

/* Same layout as recon_pose (recon_c_api.h:59-63): world->camera, R row-major. */
typedef struct orc_pose {
  double r[9];
  double t[3];
  double timestamp_ns;
} orc_pose;

/* Field-for-field image of recon::MvsConfig (core/include/recon/mvs.h:24-67);
 * bool fields are int32. */
typedef struct orc_config {
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
} orc_config;

/* The inputs of one reference view (the PatchMatchStereo argument list,
 * mvs.h:164-177), with the reference's index contract (mvs.h:151-161):
 * src / src_w / src_h use the relative index k, poses the global index
 * source_indices[k], intrinsics global when num_src_intr == num_src_poses,
 * else relative when num_src_intr == num_src. */
typedef struct orc_views {
  const uint8_t* ref;
  int32_t ref_w, ref_h;
  int32_t num_src;
  const uint8_t* const* src;
  const int32_t* src_w;
  const int32_t* src_h;
  const orc_pose* ref_pose;
  const orc_pose* src_poses;
  int32_t num_src_poses;
  const orc_intrinsics* ref_intr;
  const orc_intrinsics* src_intr;
  int32_t num_src_intr;
  const int32_t* source_indices;
  /* Optional FP32 intensities (e.g. undistorted images) read instead of the
   * 8-bit ones by orc_plane_cost and orc_plane_patchmatch; NULL = 8-bit. */
  const float* ref_f;
  const float* const* src_f;
} orc_views;

typedef struct orc_ncc_result {
  int32_t valid;
  double ncc;
  int32_t weak_texture;
  int32_t valid_samples;
} orc_ncc_result;

typedef struct orc_cost_result {
  double cost;
  double ncc_sum;
  double weight_sum;
  int32_t weak_texture_count;
  int32_t valid_views;
} orc_cost_result;

/* ---- camera model (core/src/util/camera.cpp) ---- */
void orc_apply_distortion(const orc_intrinsics* k, double x, double y, double* ox, double* oy);
void orc_remove_distortion(const orc_intrinsics* k, double xd, double yd, double* ox, double* oy);
void orc_pixel_to_ray(const orc_intrinsics* k, double u, double v, double ray[3]);
int32_t orc_project_point(const orc_intrinsics* k, const double p[3], double* u, double* v);

/* ---- core/src/mvs/patchmatch_stereo.cpp ---- */
int32_t orc_sample_bilinear(const uint8_t* img, int32_t w, int32_t h, double u, double v, double* out);
orc_ncc_result orc_compute_ncc(const uint8_t* ref, int32_t ref_w, int32_t ref_h,
                               const uint8_t* src, int32_t src_w, int32_t src_h,
                               double ref_u, double ref_v, double src_u, double src_v,
                               int32_t patch_size);
orc_cost_result orc_evaluate_candidate(const orc_views* v, const orc_config* cfg,
                                       double u, double vv, double inv_depth);
/* Batched form for tests: n hypotheses (x[i], y[i] integer pixel, inv[i]). */
void orc_evaluate_candidates(const orc_views* v, const orc_config* cfg, int32_t n,
                             const int32_t* px, const int32_t* py, const double* inv,
                             double* out_cost, int32_t* out_valid_views);

uint32_t orc_xorshift_next(uint64_t* state);

/* Contract checks + mean baseline + inverse-depth range.  Returns 0 on a
 * contract violation, else 1 with *inv_min, *inv_max, *baseline filled. */
int32_t orc_pm_prepare(const orc_views* v, const orc_config* cfg,
                       double* inv_min, double* inv_max, double* baseline);
/* Seeding + random init + initial cost (patchmatch_stereo.cpp:487-581). */
void orc_pm_init(const orc_views* v, const orc_config* cfg,
                 const double* seed_points, int32_t num_seeds,
                 double* inv, double* cost, int32_t* support);
/* One direction sweep (patchmatch_stereo.cpp:607-741) from the state
 * (inv, cost, support), writing the next state into out_*. */
void orc_pm_sweep(const orc_views* v, const orc_config* cfg, int32_t iter, int32_t dir,
                  const double* inv, const double* cost, const int32_t* support,
                  double* out_inv, double* out_cost, int32_t* out_support);
/* Output conversion (patchmatch_stereo.cpp:744-763). */
uint32_t orc_pm_output(const orc_views* v, const orc_config* cfg,
                       const double* inv, const double* cost, const int32_t* support,
                       float* depth, uint8_t* support_count, float* confidence);
uint32_t orc_patchmatch_stereo(const orc_views* v, const orc_config* cfg,
                               const double* seed_points, int32_t num_seeds,
                               float* depth, uint8_t* support_count, float* confidence);
uint32_t orc_refine_subpixel(const orc_views* v, const orc_config* cfg,
                             float* depth, uint8_t* support_count, float* confidence);
/* Per-pixel refinement of the listed pixels only (for sampled parity checks).
 * Writes the refined inverse depth / cost / written flag per listed pixel. */
void orc_refine_pixels(const orc_views* v, const orc_config* cfg, const float* depth,
                       int32_t n, const int32_t* px, const int32_t* py,
                       double* out_best_inv, double* out_best_cost, int32_t* out_written);

/* One depth map for fusion. */
typedef struct orc_depth_map {
  int32_t width, height;
  const float* depth;
  const uint8_t* support_count;
  const float* confidence;
} orc_depth_map;

/* FuseDepthMaps (patchmatch_stereo.cpp:985-1089).  Returns the voxel count.
 * Outputs (capacity max_out) are sorted by voxel key.  A NULL out_keys only
 * counts. */
int64_t orc_fuse_depth_maps(const orc_depth_map* maps, int32_t num_maps,
                            const orc_pose* poses, const orc_intrinsics* intr,
                            const orc_config* cfg, int64_t max_out,
                            int64_t* out_keys, double* out_pos, double* out_normal,
                            float* out_conf, uint32_t* out_count);

/* SelectSourceViews (patchmatch_stereo.cpp:133-211).  Returns the count. */
int32_t orc_select_source_views(const orc_pose* ref_pose, const orc_pose* poses,
                                int32_t num_poses, const orc_intrinsics* intr,
                                const orc_config* cfg, int32_t* out_indices);

/* ---------------- restatements without a reference CPU function ---------- */

/* Plane-induced homography NCC cost, FP64.  The GPU engine's "plane" cost
 * mode: hypothesis (inverse depth at the pixel centre, unit normal in the
 * reference camera frame); window samples at the reference pixel centres
 * (x+dx+0.5, y+dy+0.5) mapped through H = K_s (A + b n^T / delta) K_r^-1;
 * images read with pixel-centre convention (index = coordinate - 0.5);
 * validity rules of ComputeNcc; per-view cost 1 - NCC aggregated as the
 * mean of the best_k lowest view costs.  Pinhole only (undistorted input). */
typedef struct orc_plane_result {
  double cost;
  int32_t valid_views;
  double view_cost[32];
  int32_t view_valid[32];
  double view_edge[32]; /* per valid view: the smallest distance of a window sample to a texel edge */
} orc_plane_result;
/* half_pixel = 1 selects the reference's sampling convention instead: the
 * reference window sampled at (x+0.5+dx, y+0.5+dy) with index == coordinate
 * (SampleBilinear, patchmatch_stereo.cpp:78-100) and source coordinates used
 * as indices directly. */
orc_plane_result orc_plane_cost(const orc_views* v, const orc_config* cfg, int32_t best_k,
                                int32_t x, int32_t y, double inv_depth, const double n[3],
                                int32_t half_pixel);
void orc_plane_costs(const orc_views* v, const orc_config* cfg, int32_t best_k, int32_t n,
                     const int32_t* px, const int32_t* py, const double* inv,
                     const double* normals, double* out_cost, int32_t* out_valid_views,
                     double* out_view_cost, int32_t half_pixel);
/* Per hypothesis: the smallest distance, in texels, from a window sample of
 * the views the cost averages (the best_k lowest) to a texel edge of the
 * source image -- where bilinear interpolation has a kink, so the cost is not
 * differentiable there, and two evaluations whose sample positions differ by
 * rounding may fall on opposite sides (pixel-centre windows). */
void orc_plane_edge_distance(const orc_views* v, const orc_config* cfg, int32_t best_k, int32_t n,
                             const int32_t* px, const int32_t* py, const double* inv,
                             const double* normals, double* out_dist);

/* Plane-mode PatchMatch with every cost in FP64 (orc_plane_cost, pixel-centre
 * windows): the GPU engine's red-black search -- 8 adaptive propagation
 * regions, 5 refinement hypotheses per half-sweep, counter-based random
 * streams, golden-section refinement -- restated as the FP64 run the
 * mixed-precision forms are compared with.  depth NaN where invalid; normal
 * (optional) 3 floats per pixel; cost (optional).  Returns the filled count. */
uint32_t orc_plane_patchmatch(const orc_views* v, const orc_config* cfg, int32_t best_k, uint64_t seed,
                              int32_t refine, float* depth, float* normal, float* cost);
/* The same with prune = 1: the engine's exact shortcuts (a sweep candidate
 * stops once its views bound its cost above the pixel's; a propagation
 * candidate equal to the one just rejected is skipped).  The maps are the
 * ones prune = 0 gives. */
uint32_t orc_plane_patchmatch_ex(const orc_views* v, const orc_config* cfg, int32_t best_k, uint64_t seed,
                                 int32_t refine, int32_t prune, float* depth, float* normal, float* cost);
/* The same with the engine's exploration schedule (options.exploration_iterations):
 * explore_iters > 0 evaluates the random and fronto-parallel refinement
 * candidates only in iterations < explore_iters (they are drawn either way,
 * so the random streams are those of the full schedule); 0 = every iteration. */
uint32_t orc_plane_patchmatch_ex2(const orc_views* v, const orc_config* cfg, int32_t best_k, uint64_t seed,
                                  int32_t refine, int32_t prune, int32_t explore_iters, float* depth, float* normal,
                                  float* cost);

/* Geometric consistency (spec: shaders/vulkan/recon_mvs_consistency.comp:94-140
 * with the strict transform of shaders/common/gpu_algo.h:537-538, plus a
 * reprojection-error bound).  FP32 arithmetic in a fixed order on relative
 * transforms composed in FP64 -- the GPU kernel performs the identical IEEE
 * operation sequence, so support counts compare bit-exactly. */
typedef struct orc_consistency_params {
  float rel_depth_max;   /* |z_back - z_ref| / z_ref bound */
  float reproj_px_max;   /* reprojection distance bound, pixels */
  int32_t min_views;     /* keep when count >= min_views */
} orc_consistency_params;
void orc_geo_consistency(const orc_depth_map* maps, int32_t num_maps,
                         const orc_pose* poses, const orc_intrinsics* intr,
                         int32_t ref_index, const orc_consistency_params* p,
                         uint8_t* out_count, uint8_t* out_keep);
/* The relative transform pc_src = A pc_ref + b composed in FP64 and rounded
 * to float, as both sides use it. */
void orc_relative_transform_f32(const orc_pose* ref, const orc_pose* src, float A[9], float b[3]);

/* Undistortion remap: output pixel (i,j) of a pinhole image with the same
 * fx,fy,cx,cy reads the distorted image at ApplyDistortion of its centre
 * (camera.cpp:33-45), bilinear with pixel-centre convention; 0 outside. */
void orc_undistort(const uint8_t* img, int32_t w, int32_t h, const orc_intrinsics* k,
                   float* out);

/* BgraToGray (orchestrator.cpp:53-67): BT.601 integer weights. */
void orc_bgra_to_gray(const uint8_t* bgra, int32_t w, int32_t h, int32_t stride, uint8_t* out);

/* ---- TSDF fusion (core/src/rgbd/tsdf_fusion.cpp, tsdf_internal.h) ---- */
/* TsdfConfig (core/include/recon/tsdf_fusion.h:17-39), field for field. */
typedef struct orc_tsdf_config {
  double voxel_size_m, truncation_m, min_depth_m, max_depth_m;
  double fx, fy, cx, cy;
  double origin_x, origin_y, origin_z;
  double bbox_max_x, bbox_max_y, bbox_max_z;
  int32_t min_confidence;
} orc_tsdf_config;
/* TsdfVolume's grid dimensions (x, y, z). */
void orc_tsdf_dims(const orc_tsdf_config* cfg, int32_t dims[3]);
/* TsdfVolume::IntegrateDepthFrame on grid arrays (index (iz * ny + iy) * nx
 * + ix; tsdf starts at 1, weight at 0); w2c row-major 4 x 4.  Returns the
 * pixels fused. */
uint32_t orc_tsdf_integrate(const orc_tsdf_config* cfg, float* tsdf, float* weight, const uint16_t* depth_mm,
                            const uint8_t* confidence, int32_t width, int32_t height, const double w2c[16],
                            float depth_uncertainty_m);
/* TsdfVolume::ExtractPoints: returns the count, writes at most `cap`
 * (positions / normals 3 per point, confidence, optional voxel index). */
int64_t orc_tsdf_extract(const orc_tsdf_config* cfg, const float* tsdf, const float* weight, int64_t cap,
                         double* pos, double* nrm, float* conf, int64_t* voxel_index);

#ifdef __cplusplus
}
#endif
#endif
