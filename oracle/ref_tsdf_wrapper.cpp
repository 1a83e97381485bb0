// ref_tsdf_wrapper.cpp -- C entry points over the reference's own TSDF
// fusion sources (TEST INFRASTRUCTURE ONLY).
//
// Built by `make -C oracle ref` into oracle/_ref/libref_tsdf.so from the
// reference's unmodified core/src/rgbd/tsdf_fusion.cpp and
// core/src/rgbd/tsdf_internal.h.  ref_tsdf_run drives recon::TsdfVolume
// itself (IntegrateDepthFrame per frame, then ExtractPoints); ref_tsdf_grid
// reads the grid values through the reference's own
// tsdf_internal::IntegrateFrame with TsdfVolume's storage update
// (tsdf_fusion.cpp:91-103), since the class keeps its grid private.  Used to
// pin the C restatement (tsdf_oracle.c).
#include <cstring>
#include <vector>

#include "mvs_oracle.h"
#include "recon/tsdf_fusion.h"
#include REF_TSDF_INTERNAL  // core/src/rgbd/tsdf_internal.h

namespace {

recon::TsdfConfig ToConfig(const orc_tsdf_config& c) {
  recon::TsdfConfig o;
  o.voxel_size_m = c.voxel_size_m;
  o.truncation_m = c.truncation_m;
  o.min_depth_m = c.min_depth_m;
  o.max_depth_m = c.max_depth_m;
  o.fx = c.fx;
  o.fy = c.fy;
  o.cx = c.cx;
  o.cy = c.cy;
  o.origin_x = c.origin_x;
  o.origin_y = c.origin_y;
  o.origin_z = c.origin_z;
  o.bbox_max_x = c.bbox_max_x;
  o.bbox_max_y = c.bbox_max_y;
  o.bbox_max_z = c.bbox_max_z;
  o.min_confidence = c.min_confidence;
  return o;
}

recon::Mat4d ToMat(const double* m) {
  recon::Mat4d o;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) o(i, j) = m[i * 4 + j];
  return o;
}

}  // namespace

extern "C" int64_t ref_tsdf_run(const orc_tsdf_config* cfg, int32_t nframes, const uint16_t* depth,
                                const uint8_t* conf, int32_t w, int32_t h, const double* w2c, const float* unc,
                                uint32_t* integrated, int64_t cap, double* pos, double* nrm, float* conf_out) {
  recon::TsdfVolume vol(ToConfig(*cfg));
  const size_t n = (size_t)w * h;
  for (int f = 0; f < nframes; ++f)
    integrated[f] = vol.IntegrateDepthFrame(depth + f * n, conf ? conf + f * n : nullptr, w, h, ToMat(w2c + 16 * f),
                                            unc[f]);
  std::vector<recon::Vec3d> p, q;
  std::vector<float> c;
  vol.ExtractPoints(&p, &q, &c);
  for (size_t i = 0; i < p.size() && (int64_t)i < cap; ++i) {
    for (int k = 0; k < 3; ++k) {
      pos[3 * i + k] = p[i](k);
      nrm[3 * i + k] = q[i](k);
    }
    conf_out[i] = c[i];
  }
  return (int64_t)p.size();
}

extern "C" void ref_tsdf_grid(const orc_tsdf_config* cfg, int32_t nframes, const uint16_t* depth, const uint8_t* conf,
                              int32_t w, int32_t h, const double* w2c, const float* unc, float* tsdf, float* weight) {
  const recon::TsdfConfig c = ToConfig(*cfg);
  recon::TsdfVolume probe(c);
  const int* dims = probe.dims();
  const size_t total = (size_t)dims[0] * dims[1] * dims[2];
  for (size_t i = 0; i < total; ++i) {
    tsdf[i] = 1.0f;
    weight[i] = 0.0f;
  }
  const float voxel = static_cast<float>(c.voxel_size_m);
  const recon::Vec3d origin(static_cast<float>(c.origin_x), static_cast<float>(c.origin_y),
                            static_cast<float>(c.origin_z));
  const size_t n = (size_t)w * h;
  for (int f = 0; f < nframes; ++f) {
    recon::tsdf_internal::IntegrateFrame(
        c, origin, voxel, depth + f * n, conf ? conf + f * n : nullptr, w, h, ToMat(w2c + 16 * f), unc[f],
        [&](int ix, int iy, int iz) {
          return ix >= 0 && iy >= 0 && iz >= 0 && ix < dims[0] && iy < dims[1] && iz < dims[2];
        },
        [&](int ix, int iy, int iz, float sdf, float w_new) {
          const size_t idx = ((size_t)iz * dims[1] + iy) * dims[0] + ix;
          const float w_old = weight[idx];
          const float w_sum = w_old + w_new;
          if (w_sum > 0.0f) {
            tsdf[idx] = (w_old * tsdf[idx] + w_new * sdf) / w_sum;
            weight[idx] = w_sum;
          }
        });
  }
}
