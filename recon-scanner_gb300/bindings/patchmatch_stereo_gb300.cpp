// patchmatch_stereo_gb300.cpp -- the reference-side binding.
//
// A maintainer of kai3934908500/recon-scanner drops this file into
// core/src/mvs/ in place of patchmatch_stereo.cpp and links
// librecon_mvs_gb300.so: the five MVS functions of core/include/recon/mvs.h
// keep their exact signatures and behaviour (index contract, return 0 on a
// contract violation, DepthMap (re)allocation), and run on the GB300 engine.
// Callers (Orchestrator::StageMvs, tests/unit/test_mvs.cpp) are unchanged.
//
// The search model defaults to the engine's plane mode; RECON_MVS_MODE=compat
// in the environment selects the reference's own search (translated windows,
// Jacobi sweeps, identical draws), e.g. for the reference unit test's
// expectations on fronto-parallel scenes.
#include <array>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "recon/mvs.h"
#include "recon/recon_c_api.h"  // first: recon_mvs_gb300.h reuses its types
#include "recon_mvs_gb300.h"

namespace recon {
namespace {

recon_camera_intrinsics ToC(const CameraIntrinsics& k) {
  return recon_camera_intrinsics{k.fx, k.fy, k.cx, k.cy, k.k1, k.k2, k.k3, k.p1, k.p2,
                                 static_cast<double>(k.width), static_cast<double>(k.height)};
}

recon_pose ToC(const CameraPose& p) {
  recon_pose o;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) o.r[i * 3 + j] = p.R(i, j);
  for (int i = 0; i < 3; ++i) o.t[i] = p.t(i);
  o.timestamp_ns = 0.0;
  return o;
}

recon_mvs_config ToC(const MvsConfig& c) {
  recon_mvs_config o;
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
  o.propagation_enabled = c.propagation_enabled ? 1 : 0;
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

recon_mvs_options Options() {
  recon_mvs_options o;
  recon_mvs_options_default(&o);
  const char* m = std::getenv("RECON_MVS_MODE");
  if (m && std::strcmp(m, "compat") == 0) o.mode = RECON_MVS_MODE_COMPAT;
  return o;
}

struct ViewsC {
  std::vector<recon_pose> poses;
  std::vector<recon_camera_intrinsics> intr;
  std::vector<int32_t> w, h, idx;
  recon_pose ref_pose;
  recon_camera_intrinsics ref_intr;
  recon_mvs_views v;
};

void Fill(ViewsC* c, const uint8_t* ref_gray, int ref_w, int ref_h, const std::vector<const uint8_t*>& src_gray,
          const std::vector<int>& src_w, const std::vector<int>& src_h, const CameraPose& ref_pose,
          const std::vector<CameraPose>& src_poses, const CameraIntrinsics& ref_intr,
          const std::vector<CameraIntrinsics>& src_intrinsics, const std::vector<int>& source_indices) {
  for (const auto& p : src_poses) c->poses.push_back(ToC(p));
  for (const auto& k : src_intrinsics) c->intr.push_back(ToC(k));
  c->w.assign(src_w.begin(), src_w.end());
  c->h.assign(src_h.begin(), src_h.end());
  c->idx.assign(source_indices.begin(), source_indices.end());
  c->ref_pose = ToC(ref_pose);
  c->ref_intr = ToC(ref_intr);
  c->v = recon_mvs_views{ref_gray, ref_w, ref_h, static_cast<int32_t>(source_indices.size()),
                         src_gray.data(), c->w.data(), c->h.data(), &c->ref_pose, c->poses.data(),
                         static_cast<int32_t>(c->poses.size()), &c->ref_intr, c->intr.data(),
                         static_cast<int32_t>(c->intr.size()), c->idx.data()};
  // the reference checks the sizes of these arrays against source_indices
  if (src_gray.size() != source_indices.size() || src_w.size() != source_indices.size() ||
      src_h.size() != source_indices.size())
    c->v.num_src = -1;
}

}  // namespace

std::vector<int> SelectSourceViews(const CameraPose& ref_pose, const std::vector<CameraPose>& poses,
                                   const CameraIntrinsics& intrinsics, const MvsConfig& config) {
  std::vector<recon_pose> ps;
  for (const auto& p : poses) ps.push_back(ToC(p));
  const recon_pose rp = ToC(ref_pose);
  const recon_camera_intrinsics k = ToC(intrinsics);
  const recon_mvs_config c = ToC(config);
  std::vector<int32_t> out(poses.size() + 1);
  int32_t n = 0;
  if (recon_mvs_select_source_views(&rp, ps.data(), static_cast<int32_t>(ps.size()), &k, &c, out.data(),
                                    static_cast<int32_t>(out.size()), &n) != RECON_OK)
    return {};
  return std::vector<int>(out.begin(), out.begin() + n);
}

NccResult ComputeNcc(const uint8_t* ref_img, int ref_w, int ref_h, const uint8_t* src_img, int src_w, int src_h,
                     double ref_u, double ref_v, double src_u, double src_v, int patch_size) {
  const double coords[4] = {ref_u, ref_v, src_u, src_v};
  recon_mvs_ncc_result r{};
  NccResult out;
  if (recon_mvs_compute_ncc(ref_img, ref_w, ref_h, src_img, src_w, src_h, coords, 1, patch_size, &r) != RECON_OK)
    return out;
  out.valid = r.valid != 0;
  out.ncc = r.ncc;
  out.weak_texture = r.weak_texture != 0;
  out.valid_samples = r.valid_samples;
  return out;
}

uint32_t PatchMatchStereo(const uint8_t* ref_gray, int ref_w, int ref_h, const std::vector<const uint8_t*>& src_gray,
                          const std::vector<int>& src_w, const std::vector<int>& src_h, const CameraPose& ref_pose,
                          const std::vector<CameraPose>& src_poses, const CameraIntrinsics& ref_intr,
                          const std::vector<CameraIntrinsics>& src_intrinsics, const std::vector<int>& source_indices,
                          const MvsConfig& config, const std::vector<std::array<double, 3>>* seed_points,
                          DepthMap* out_depth) {
  if (ref_gray == nullptr || out_depth == nullptr || source_indices.empty()) return 0;
  ViewsC c;
  Fill(&c, ref_gray, ref_w, ref_h, src_gray, src_w, src_h, ref_pose, src_poses, ref_intr, src_intrinsics,
       source_indices);
  if (c.v.num_src < 0) return 0;
  const recon_mvs_config cfg = ToC(config);
  const recon_mvs_options opts = Options();
  std::vector<double> seeds;
  if (seed_points)
    for (const auto& s : *seed_points) seeds.insert(seeds.end(), s.begin(), s.end());
  DepthMap tmp;
  tmp.Allocate(ref_w, ref_h);
  recon_mvs_depth_map dm{ref_w, ref_h, tmp.depth.data(), tmp.support_count.data(), tmp.confidence.data(), nullptr,
                         nullptr};
  uint32_t filled = 0;
  const recon_status st = recon_mvs_patchmatch(&c.v, &cfg, &opts, seeds.empty() ? nullptr : seeds.data(),
                                               static_cast<int32_t>(seeds.size() / 3), &dm, &filled);
  if (st != RECON_OK) return 0;  // the reference returns 0 on a contract violation
  *out_depth = std::move(tmp);
  return filled;
}

uint32_t RefineSubpixel(const uint8_t* ref_gray, int ref_w, int ref_h, const std::vector<const uint8_t*>& src_gray,
                        const std::vector<int>& src_w, const std::vector<int>& src_h, const CameraPose& ref_pose,
                        const std::vector<CameraPose>& src_poses, const CameraIntrinsics& ref_intr,
                        const std::vector<CameraIntrinsics>& src_intrinsics, const std::vector<int>& source_indices,
                        const MvsConfig& config, DepthMap* depth) {
  if (ref_gray == nullptr || depth == nullptr || source_indices.empty()) return 0;
  if (depth->width != ref_w || depth->height != ref_h) return 0;
  ViewsC c;
  Fill(&c, ref_gray, ref_w, ref_h, src_gray, src_w, src_h, ref_pose, src_poses, ref_intr, src_intrinsics,
       source_indices);
  if (c.v.num_src < 0) return 0;
  const recon_mvs_config cfg = ToC(config);
  recon_mvs_depth_map dm{ref_w, ref_h, depth->depth.data(), depth->support_count.data(), depth->confidence.data(),
                         nullptr, nullptr};
  uint32_t refined = 0;
  if (recon_mvs_refine_subpixel(&c.v, &cfg, nullptr, &dm, &refined) != RECON_OK) return 0;
  return refined;
}

PointCloud FuseDepthMaps(const std::vector<const DepthMap*>& depth_maps, const std::vector<CameraPose>& poses,
                         const std::vector<CameraIntrinsics>& intrinsics, const MvsConfig& config) {
  PointCloud cloud;
  std::vector<recon_mvs_depth_map> maps;
  std::vector<recon_pose> ps;
  std::vector<recon_camera_intrinsics> ks;
  for (size_t i = 0; i < depth_maps.size(); ++i) {
    const DepthMap* d = depth_maps[i];
    maps.push_back(d ? recon_mvs_depth_map{d->width, d->height, const_cast<float*>(d->depth.data()),
                                           const_cast<uint8_t*>(d->support_count.data()),
                                           const_cast<float*>(d->confidence.data()), nullptr, nullptr}
                     : recon_mvs_depth_map{0, 0, nullptr, nullptr, nullptr, nullptr, nullptr});
    ps.push_back(ToC(poses[i]));
    ks.push_back(ToC(intrinsics[i]));
  }
  const recon_mvs_config cfg = ToC(config);
  recon_mvs_point_cloud pc{};
  if (recon_mvs_fuse(maps.data(), ps.data(), ks.data(), static_cast<int32_t>(maps.size()), &cfg, nullptr, &pc) !=
      RECON_OK)
    return cloud;
  for (int64_t i = 0; i < pc.count; ++i) {
    cloud.positions.push_back(Vec3d(pc.positions[3 * i], pc.positions[3 * i + 1], pc.positions[3 * i + 2]));
    cloud.normals.push_back(Vec3d(pc.normals[3 * i], pc.normals[3 * i + 1], pc.normals[3 * i + 2]));
    cloud.confidences.push_back(pc.confidences[i]);
    for (int q = 0; q < 3; ++q) cloud.colors.push_back(pc.colors[3 * i + q]);
  }
  recon_mvs_point_cloud_free(&pc);
  return cloud;
}

}  // namespace recon
