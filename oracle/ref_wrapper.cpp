// ref_wrapper.cpp -- C entry points over the reference's own MVS sources.
//
// TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle ref` (and by build()
// when the reference tree is present) into oracle/_ref/libref_mvs.so, straight
// from the reference's unmodified sources, which this translation unit
// includes by path so that the anonymous-namespace EvaluateCandidate of
// core/src/mvs/patchmatch_stereo.cpp is reachable.  It is used to pin the C
// restatement (mvs_oracle.c) with golden vectors, and as the timed reference
// CPU baseline where it exists.
//
// The entry points take the same POD structs as the restatement
// (mvs_oracle.h), so one Python loader drives both.

#include REF_PM_SOURCE  // core/src/mvs/patchmatch_stereo.cpp

#include <cstring>

#include "mvs_oracle.h"

namespace {

recon::CameraIntrinsics ToIntr(const orc_intrinsics& k) {
  recon::CameraIntrinsics o;
  o.fx = k.fx;
  o.fy = k.fy;
  o.cx = k.cx;
  o.cy = k.cy;
  o.k1 = k.k1;
  o.k2 = k.k2;
  o.k3 = k.k3;
  o.p1 = k.p1;
  o.p2 = k.p2;
  o.width = static_cast<int>(k.width);
  o.height = static_cast<int>(k.height);
  return o;
}

recon::CameraPose ToPose(const orc_pose& p) {
  recon::CameraPose o;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o.R(i, j) = p.r[i * 3 + j];
  for (int i = 0; i < 3; ++i) o.t(i) = p.t[i];
  return o;
}

recon::MvsConfig ToConfig(const orc_config& c) {
  recon::MvsConfig o;
  o.num_views = c.num_views;
  o.ref_view_index = c.ref_view_index;
  o.ideal_angle_min_deg = c.ideal_angle_min_deg;
  o.ideal_angle_max_deg = c.ideal_angle_max_deg;
  o.max_view_scale_mismatch = c.max_view_scale_mismatch;
  o.view_angle_weight = c.view_angle_weight;
  o.view_texture_weight = c.view_texture_weight;
  o.view_spread_weight = c.view_spread_weight;
  o.view_scale_weight = c.view_scale_weight;
  o.reference_depth_m = c.reference_depth_m;
  o.patch_size = c.patch_size;
  o.iterations = c.iterations;
  o.random_search_count = c.random_search_count;
  o.random_search_radius_ratio = c.random_search_radius_ratio;
  o.restart_ratio = c.restart_ratio;
  o.propagation_directions = c.propagation_directions;
  o.propagation_enabled = c.propagation_enabled != 0;
  o.num_threads = c.num_threads;
  o.photo_threshold = c.photo_threshold;
  o.depth_regularization = c.depth_regularization;
  o.geo_consistency_threshold = c.geo_consistency_threshold;
  o.weak_texture_variance = c.weak_texture_variance;
  o.subpixel_iterations = c.subpixel_iterations;
  o.subpixel_fit_points = c.subpixel_fit_points;
  o.subpixel_window_ratio = c.subpixel_window_ratio;
  o.min_depth_m = c.min_depth_m;
  o.max_depth_m = c.max_depth_m;
  o.min_view_consistency = c.min_view_consistency;
  o.fusion_voxel_size_m = c.fusion_voxel_size_m;
  return o;
}

struct Args {
  std::vector<const uint8_t*> src;
  std::vector<int> src_w, src_h;
  recon::CameraPose ref_pose;
  std::vector<recon::CameraPose> poses;
  recon::CameraIntrinsics ref_intr;
  std::vector<recon::CameraIntrinsics> intr;
  std::vector<int> idx;
  bool global = false;
};

Args ToArgs(const orc_views* v) {
  Args a;
  for (int k = 0; k < v->num_src; ++k) {
    a.src.push_back(v->src[k]);
    a.src_w.push_back(v->src_w[k]);
    a.src_h.push_back(v->src_h[k]);
    a.idx.push_back(v->source_indices[k]);
  }
  a.ref_pose = ToPose(*v->ref_pose);
  for (int i = 0; i < v->num_src_poses; ++i) a.poses.push_back(ToPose(v->src_poses[i]));
  a.ref_intr = ToIntr(*v->ref_intr);
  for (int i = 0; i < v->num_src_intr; ++i) a.intr.push_back(ToIntr(v->src_intr[i]));
  a.global = (a.intr.size() == a.poses.size());
  return a;
}

}  // namespace

extern "C" {

void ref_pixel_to_ray(const orc_intrinsics* k, double u, double v, double ray[3]) {
  recon::Vec3d r;
  ToIntr(*k).PixelToRay(u, v, &r);
  for (int i = 0; i < 3; ++i) ray[i] = r(i);
}

int32_t ref_project_point(const orc_intrinsics* k, const double p[3], double* u, double* v) {
  return ToIntr(*k).ProjectPoint(recon::Vec3d(p[0], p[1], p[2]), u, v) ? 1 : 0;
}

orc_ncc_result ref_compute_ncc(const uint8_t* ref, int32_t ref_w, int32_t ref_h, const uint8_t* src,
                               int32_t src_w, int32_t src_h, double ref_u, double ref_v,
                               double src_u, double src_v, int32_t patch_size) {
  const recon::NccResult r = recon::ComputeNcc(ref, ref_w, ref_h, src, src_w, src_h, ref_u, ref_v,
                                               src_u, src_v, patch_size);
  orc_ncc_result o;
  o.valid = r.valid;
  o.ncc = r.ncc;
  o.weak_texture = r.weak_texture;
  o.valid_samples = r.valid_samples;
  return o;
}

void ref_evaluate_candidates(const orc_views* v, const orc_config* cfg, int32_t n, const int32_t* px,
                             const int32_t* py, const double* inv, double* out_cost,
                             int32_t* out_valid_views) {
  const Args a = ToArgs(v);
  const recon::MvsConfig c = ToConfig(*cfg);
  for (int32_t i = 0; i < n; ++i) {
    const recon::CostResult r = recon::EvaluateCandidate(
        px[i] + 0.5, py[i] + 0.5, inv[i], v->ref, v->ref_w, v->ref_h, a.src, a.src_w, a.src_h,
        a.ref_pose, a.poses, a.ref_intr, a.intr, a.idx, c, a.global);
    out_cost[i] = r.cost;
    out_valid_views[i] = r.valid_views;
  }
}

uint32_t ref_patchmatch_stereo(const orc_views* v, const orc_config* cfg, const double* seeds,
                               int32_t num_seeds, float* depth, uint8_t* support, float* conf) {
  const Args a = ToArgs(v);
  const recon::MvsConfig c = ToConfig(*cfg);
  std::vector<std::array<double, 3>> sp;
  for (int i = 0; i < num_seeds; ++i) sp.push_back({seeds[3 * i], seeds[3 * i + 1], seeds[3 * i + 2]});
  recon::DepthMap dm;
  const uint32_t filled = recon::PatchMatchStereo(v->ref, v->ref_w, v->ref_h, a.src, a.src_w, a.src_h,
                                                  a.ref_pose, a.poses, a.ref_intr, a.intr, a.idx, c,
                                                  num_seeds > 0 ? &sp : nullptr, &dm);
  if (dm.width == v->ref_w && dm.height == v->ref_h) {
    std::memcpy(depth, dm.depth.data(), dm.depth.size() * sizeof(float));
    std::memcpy(support, dm.support_count.data(), dm.support_count.size());
    std::memcpy(conf, dm.confidence.data(), dm.confidence.size() * sizeof(float));
  }
  return filled;
}

uint32_t ref_refine_subpixel(const orc_views* v, const orc_config* cfg, float* depth, uint8_t* support,
                             float* conf) {
  const Args a = ToArgs(v);
  const recon::MvsConfig c = ToConfig(*cfg);
  recon::DepthMap dm;
  dm.width = v->ref_w;
  dm.height = v->ref_h;
  const size_t n = static_cast<size_t>(v->ref_w) * v->ref_h;
  dm.depth.assign(depth, depth + n);
  dm.support_count.assign(support, support + n);
  dm.confidence.assign(conf, conf + n);
  const uint32_t refined = recon::RefineSubpixel(v->ref, v->ref_w, v->ref_h, a.src, a.src_w, a.src_h,
                                                 a.ref_pose, a.poses, a.ref_intr, a.intr, a.idx, c, &dm);
  std::memcpy(depth, dm.depth.data(), n * sizeof(float));
  std::memcpy(conf, dm.confidence.data(), n * sizeof(float));
  return refined;
}

int64_t ref_fuse_depth_maps(const orc_depth_map* maps, int32_t num_maps, const orc_pose* poses,
                            const orc_intrinsics* intr, const orc_config* cfg, int64_t max_out,
                            double* out_pos, double* out_normal, float* out_conf) {
  std::vector<recon::DepthMap> dms(static_cast<size_t>(num_maps));
  std::vector<const recon::DepthMap*> ptrs;
  std::vector<recon::CameraPose> ps;
  std::vector<recon::CameraIntrinsics> ks;
  for (int i = 0; i < num_maps; ++i) {
    const size_t n = static_cast<size_t>(maps[i].width) * maps[i].height;
    dms[i].width = maps[i].width;
    dms[i].height = maps[i].height;
    dms[i].depth.assign(maps[i].depth, maps[i].depth + n);
    dms[i].support_count.assign(maps[i].support_count, maps[i].support_count + n);
    dms[i].confidence.assign(maps[i].confidence, maps[i].confidence + n);
    ptrs.push_back(&dms[i]);
    ps.push_back(ToPose(poses[i]));
    ks.push_back(ToIntr(intr[i]));
  }
  const recon::PointCloud pc = recon::FuseDepthMaps(ptrs, ps, ks, ToConfig(*cfg));
  const int64_t total = static_cast<int64_t>(pc.size());
  for (int64_t i = 0; i < total && i < max_out; ++i) {
    for (int q = 0; q < 3; ++q) out_pos[3 * i + q] = pc.positions[i](q);
    for (int q = 0; q < 3; ++q) out_normal[3 * i + q] = pc.normals[i](q);
    out_conf[i] = pc.confidences[i];
  }
  return total;
}

int32_t ref_select_source_views(const orc_pose* ref_pose, const orc_pose* poses, int32_t num_poses,
                                const orc_intrinsics* intr, const orc_config* cfg,
                                int32_t* out_indices) {
  std::vector<recon::CameraPose> ps;
  for (int i = 0; i < num_poses; ++i) ps.push_back(ToPose(poses[i]));
  const std::vector<int> sel =
      recon::SelectSourceViews(ToPose(*ref_pose), ps, ToIntr(*intr), ToConfig(*cfg));
  for (size_t i = 0; i < sel.size(); ++i) out_indices[i] = sel[i];
  return static_cast<int32_t>(sel.size());
}

}  // extern "C"
