// kernels.h -- launch interface between the host runtime (engine.cu) and
// the kernels (pm.cu, fusion.cu).  Internal to the library.
#pragma once

#include <cuda_fp16.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "common.cuh"
#include "recon_mvs_gb300.h"

namespace rmvs {

// ---- fusion / consistency / undistortion descriptors ----
struct FuseMap {
  int w, h;
  const float* depth;
  const uint8_t* support;
  const float* conf;
  const uint8_t* keep;  // optional consistency mask
  const float* normal;  // optional camera-frame unit normals (3 per pixel): fused instead of -ray
  double fx, fy, cx, cy, k1, k2, k3, p1, p2;
  double R[9], t[3];
};

struct FuseParams {
  double voxel;
  double photo_threshold;
  int min_view_consistency;
};

struct ConsistencyRef {
  int w, h;
  const float* depth;
  float fx, fy, cx, cy;
};

struct ConsistencySrc {
  int w, h;
  const float* depth;
  float fx, fy, cx, cy;
  float A[9], b[3];    // reference camera -> this camera
  float Ai[9], bi[3];  // this camera -> reference camera
};

// X_src = A X_ref + b with A = R_src R_ref^T and b = t_src - A t_ref, in FP64
// and in this operation order: consistency counts and fused clouds are
// compared bit for bit with the oracle, which composes the same way.  Every
// caller (the allocating and the allocation-free consistency entry points,
// the plane-mode job set-up) shares this one definition.
inline void relative_transform(const recon_pose& ref, const recon_pose& src, double A[9], double b[3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int q = 0; q < 3; ++q) s += src.r[i * 3 + q] * ref.r[j * 3 + q];
      A[i * 3 + j] = s;
    }
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += A[i * 3 + j] * ref.t[j];
    b[i] = src.t[i] - s;
  }
}

// The consistency descriptor of one source map seen from the reference pose.
inline ConsistencySrc consistency_source(int w, int h, const float* depth, const recon_camera_intrinsics& intr,
                                         const recon_pose& ref_pose, const recon_pose& src_pose) {
  ConsistencySrc cs;
  memset(&cs, 0, sizeof(cs));
  cs.w = w;
  cs.h = h;
  cs.depth = depth;
  cs.fx = (float)intr.fx;
  cs.fy = (float)intr.fy;
  cs.cx = (float)intr.cx;
  cs.cy = (float)intr.cy;
  double A[9], b[3], Ai[9], bi[3];
  relative_transform(ref_pose, src_pose, A, b);
  relative_transform(src_pose, ref_pose, Ai, bi);
  for (int i = 0; i < 9; ++i) {
    cs.A[i] = (float)A[i];
    cs.Ai[i] = (float)Ai[i];
  }
  for (int i = 0; i < 3; ++i) {
    cs.b[i] = (float)b[i];
    cs.bi[i] = (float)bi[i];
  }
  return cs;
}

struct UndistortCam {
  double fx, fy, cx, cy, k1, k2, k3, p1, p2;
};

struct NccWindow {
  double ref_u, ref_v, src_u, src_v;
};

// ---- PatchMatch ----
cudaError_t launch_eval_hyps(const Job& J, int mode, int n, const int* px, const int* py, const double* inv,
                             const float* normals, float* cost, int* support, float* view_cost, cudaStream_t st);
// Plane-mode batches.  A batch's work items are tiles of its jobs, listed
// job after job; start[j] is the first item of job j and start[njobs] the
// batch's item count.  Pixel-tile kernels (init, refine, output) use 32 x 4
// pixel tiles; sweeps use 64-column x rows tiles with their own prefix.  The
// whole record is a kernel parameter (<= 32 KB): the jobs sit in the
// constant bank.
constexpr int kMaxTileRows = 8;
constexpr int kBatchJobs = 64;
struct PlaneBatch {
  Job jobs[kBatchJobs];
  int start[kBatchJobs + 1];
  int njobs;
  // sweeps: one TMA tensor map per job over its ref_de planes (device memory,
  // 64-byte aligned), box = kTileCols columns x (rows + 2H) rows x 2 planes
  const CUtensorMap* tmaps;
  int* err;  // set when a TMA wait runs out (the launch then stops early)
  // fault injection for the test of that path: 1 = issue no tile copy (every
  // wait runs out); the poll limit of a wait (0 = the default)
  int tma_skip;
  int tma_poll_limit;
};
static_assert(sizeof(PlaneBatch) + 64 <= 32764, "PlaneBatch exceeds the kernel-parameter limit");
cudaError_t launch_plane_init(const PlaneBatch& B, int patch_half, int mode, int max_src, int* queues, int num_queues,
                              cudaStream_t st);
// `staged` = 1: the staged-window schedule of the sweep (exact interpolation,
// 7x7 or 11x11 windows, every source with a pair map): per (candidate, view)
// a warp copies the source box its windows cover into shared memory by TMA
// and samples it there; windows whose warp footprint does not fit read the
// texture.  The maps are the same either way.
cudaError_t plane_sweep_occupancy(int patch_half, int mode, int max_src, int rows, int staged, int* blocks_per_sm);
cudaError_t launch_plane_sweep(const PlaneBatch& B, int total, int* queue, int patch_half, int mode, int max_src,
                               int rows, int staged, int grid, int color, int iter, cudaStream_t st);
// The texel-pair image of a source texture (the staged-window schedule's
// TMA source): out[y * pitch + x] = {T(x, y), T(x + 1, y)}, the second word
// 0 in the last column.
cudaError_t launch_pair_image(cudaTextureObject_t tex, int w, int h, float2* out, int pitch, cudaStream_t st);
cudaError_t launch_plane_refine(const PlaneBatch& B, int patch_half, int mode, int max_src, cudaStream_t st);
cudaError_t launch_plane_refine_gn(const PlaneBatch& B, int patch_half, int mode, int max_src, cudaStream_t st);
cudaError_t launch_plane_output(const PlaneBatch& B, cudaStream_t st);

// ---- the differentiation form (adjoint.cu) ----
// Per hypothesis (pixel, depth, theta / phi): cost, gradient (d, theta, phi),
// Gauss-Newton matrix (6, upper triangle; optional), pose gradient
// (num_src x 6: rotation, translation; optional).
cudaError_t launch_plane_adjoint(const Job& J, int n, const int* px, const int* py, const double* depth,
                                 const double* angles, float* cost, float* grad, float* gn, float* pose_grad,
                                 cudaStream_t st);
// Pose normal equations: per (block, source) records of pose_partial_records()
// floats: cost sum, gradient (6), Gauss-Newton matrix (21), pixel count.
int pose_partial_records();
cudaError_t launch_pose_normal_eq(const Job& J, int n, const int* px, const int* py, const double* depth,
                                  const double* angles, float* partial, cudaStream_t st);

cudaError_t launch_compat_init(const Job& J, float* cost, cudaStream_t st);
cudaError_t launch_compat_sweep(const Job& J, const double* inv_in, const float* cost_in, const int32_t* sup_in,
                                double* inv_out, float* cost_out, int32_t* sup_out, const uint32_t* draws,
                                const uint8_t* fire, int draw_stride, int search_count, double radius_ratio,
                                int propagate, cudaStream_t st);
cudaError_t launch_compat_output(const Job& J, const double* inv, const float* cost, const int32_t* sup, float* depth,
                                 uint8_t* support, float* conf, unsigned int* filled, cudaStream_t st);
cudaError_t launch_compat_refine(const Job& J, float* depth, float* conf, double inv_per_px, int fit_points, int iters,
                                 unsigned int* refined, double* best_inv, float* best_cost, cudaStream_t st);
cudaError_t launch_prep_ref(const uint8_t* img, int w, int h, float* ref, float* box, cudaStream_t st);
cudaError_t launch_prep_ref_f32(const float* img, int w, int h, float* ref, float* box, cudaStream_t st);
cudaError_t launch_prep_src(const uint8_t* img, int w, int h, void* out, size_t pitch_bytes, int storage,
                            cudaStream_t st);
cudaError_t launch_prep_src_f32in(const float* img, int w, int h, void* out, size_t pitch_bytes, int storage,
                                  cudaStream_t st);
cudaError_t launch_bgra_to_gray(const uint8_t* bgra, int w, int h, uint8_t* out, cudaStream_t st);
cudaError_t launch_deinterleave(const float* ref, int w, int h, int half_w, int pitch, float* out, cudaStream_t st);
cudaError_t launch_ncc_windows(const uint8_t* ref, int ref_w, int ref_h, const uint8_t* src, int src_w, int src_h,
                               int patch_size, int n, const NccWindow* win, int* valid, double* ncc, int* weak,
                               int* samples, cudaStream_t st);

// pyramid level 1 of a staged image (w / 2 x h / 2 FP32 means of 2 x 2 blocks)
cudaError_t launch_half_level(const uint8_t* in_u8, const float* in_f32, int w, int h, float* out, cudaStream_t st);
// ---- fusion ----
cudaError_t launch_cloud_finish(const double* pos, const float* conf, unsigned int n, float* weights, double* bounds,
                                cudaStream_t st);
cudaError_t launch_fuse_points(const FuseMap& M, int64_t base, const FuseParams& P, unsigned long long* key,
                               double* pos, double* nrm, float* conf, uint8_t* valid, cudaStream_t st);
cudaError_t launch_fuse_insert(int64_t n, const unsigned long long* key, const uint8_t* valid,
                               unsigned long long* tkey, unsigned int* tcount, unsigned long long* tfirst,
                               uint64_t mask, int* slot_of, int* error, cudaStream_t st);
cudaError_t launch_fuse_flags(int64_t n, const uint8_t* valid, const int* slot_of, const unsigned long long* tfirst,
                              unsigned int* flag, cudaStream_t st);
cudaError_t launch_fuse_voxels(int64_t n, const unsigned int* flag, const unsigned int* vid_of, const int* slot_of,
                               const unsigned int* tcount, unsigned int* slot_vid, unsigned int* vcount,
                               cudaStream_t st);
cudaError_t launch_fuse_scatter(int64_t n, const uint8_t* valid, const int* slot_of, const unsigned int* slot_vid,
                                const unsigned int* voffset, unsigned int* cursor, int64_t* bucket, cudaStream_t st);
cudaError_t launch_fuse_reduce(unsigned int nvox, const unsigned int* voffset, const unsigned int* vcount,
                               int64_t* bucket, const unsigned long long* key, const double* pos, const double* nrm,
                               const float* conf, unsigned long long* okey, double* opos, double* onrm, float* oconf,
                               unsigned int* ocount, cudaStream_t st);
cudaError_t launch_consistency(const ConsistencyRef& R, const ConsistencySrc* S, int num_src, float rel_max,
                               float reproj_px_max, int min_views, uint8_t* count, uint8_t* keep, cudaStream_t st);
cudaError_t launch_binomial(const uint8_t* in_u8, const float* in_f32, int w, int h, float* out, cudaStream_t st);
cudaError_t launch_undistort(const uint8_t* img, int w, int h, const UndistortCam& K, float* out, cudaStream_t st);

int64_t scan_scratch_elems(int64_t n);
cudaError_t exclusive_scan_u32(const unsigned int* in, unsigned int* out, int64_t n, unsigned int* scratch,
                               cudaStream_t st);

}  // namespace rmvs
