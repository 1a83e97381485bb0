/* tsdf_oracle.c -- CPU restatement of the reference's TSDF fusion (TEST
 * INFRASTRUCTURE ONLY).
 *
 * Follows core/src/rgbd/tsdf_fusion.cpp (TsdfVolume) and
 * core/src/rgbd/tsdf_internal.h (IntegrateFrame, SurfaceGradient) step for
 * step, with the reference's FP64 / FP32 operation order (linalg.h matrix
 * products accumulate from 0.0 over the inner index), so that, compiled with
 * -ffp-contract=off, grids and extracted points match the reference's own
 * code bit for bit.  Used only by tests/ and the bench's CPU baseline. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mvs_oracle.h"

/* FloorToIntScaled (tsdf_internal.h:32-34): floor(a / b) in FP32. */
static int floor_scaled(float a, float b) { return (int)floorf(a / b); }

static int dim_of(double bbox_max, float origin, float voxel) {
  const int n = floor_scaled((float)(bbox_max - (double)origin), voxel) + 1;
  return n > 1 ? n : 1;
}

/* TsdfVolume::TsdfVolume (tsdf_fusion.cpp:30-57): grid dimensions. */
void orc_tsdf_dims(const orc_tsdf_config* c, int32_t dims[3]) {
  const float voxel = (float)c->voxel_size_m;
  dims[0] = dim_of(c->bbox_max_x, (float)c->origin_x, voxel);
  dims[1] = dim_of(c->bbox_max_y, (float)c->origin_y, voxel);
  dims[2] = dim_of(c->bbox_max_z, (float)c->origin_z, voxel);
}

/* 3x3 matrix times vector, linalg.h:242-250 order. */
static void mat3_vec(const double m[9], const double v[3], double out[3]) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += m[i * 3 + j] * v[j];
    out[i] = s;
  }
}

/* Vec::normalized (linalg.h:71-77). */
static void normalized(const double v[3], double out[3]) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s += v[i] * v[i];
  const double n = sqrt(s);
  if (n < 1e-15) {
    out[0] = out[1] = out[2] = 0.0;
    return;
  }
  for (int i = 0; i < 3; ++i) out[i] = v[i] / n;
}

/* IntegrateFrame (tsdf_internal.h:44-143) with TsdfVolume's write
 * (tsdf_fusion.cpp:91-103): grid arrays `tsdf` (initially 1) and `weight`
 * (initially 0), index (iz * ny + iy) * nx + ix.  Returns the pixels fused. */
uint32_t orc_tsdf_integrate(const orc_tsdf_config* cfg, float* tsdf, float* weight, const uint16_t* depth_mm,
                            const uint8_t* confidence, int32_t width, int32_t height, const double w2c[16],
                            float depth_uncertainty_m) {
  if (depth_mm == NULL || width <= 0 || height <= 0) return 0u;
  const float voxel = (float)cfg->voxel_size_m;
  if (voxel <= 0.0f) return 0u;
  const float trunc = (float)cfg->truncation_m;
  if (trunc <= 0.0f) return 0u;
  int32_t dims[3];
  orc_tsdf_dims(cfg, dims);
  const double origin[3] = {(double)(float)cfg->origin_x, (double)(float)cfg->origin_y,
                            (double)(float)cfg->origin_z};
  double R_wc[9], t_wc[3], R_cw[9], t_cw[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) R_wc[i * 3 + j] = w2c[i * 4 + j];
    t_wc[i] = w2c[i * 4 + 3];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R_cw[j * 3 + i] = R_wc[i * 3 + j];
  double rt[3];
  mat3_vec(R_cw, t_wc, rt);
  for (int i = 0; i < 3; ++i) t_cw[i] = -rt[i];
  const double sig = (double)depth_uncertainty_m;
  const double sigma = sig > 1e-4 ? sig : 1e-4;
  const float w_new = (float)(1.0 / (sigma * sigma));
  const int steps = (int)(trunc / voxel) + 1;
  uint32_t integrated = 0;
  for (int v = 0; v < height; ++v) {
    for (int u = 0; u < width; ++u) {
      const size_t pix = (size_t)v * width + u;
      const uint16_t d_raw = depth_mm[pix];
      if (d_raw == 0) continue;
      if (confidence != NULL && confidence[pix] < cfg->min_confidence) continue;
      const double dx = ((double)u - cfg->cx) / cfg->fx;
      const double dy = ((double)v - cfg->cy) / cfg->fy;
      const double d_axis_m = (double)d_raw * 1e-3;
      if (d_axis_m < cfg->min_depth_m || d_axis_m > cfg->max_depth_m) continue;
      const double p_cam[3] = {dx * d_axis_m, dy * d_axis_m, d_axis_m};
      double pw[3], p_world[3];
      mat3_vec(R_cw, p_cam, pw);
      for (int i = 0; i < 3; ++i) p_world[i] = pw[i] + t_cw[i];
      double ray_cam[3], rw[3], normal_world[3];
      normalized(p_cam, ray_cam);
      mat3_vec(R_cw, ray_cam, rw);
      normalized(rw, normal_world);
      const int cx_v = floor_scaled((float)(p_world[0] - origin[0]), voxel);
      const int cy_v = floor_scaled((float)(p_world[1] - origin[1]), voxel);
      const int cz_v = floor_scaled((float)(p_world[2] - origin[2]), voxel);
      const float nx_w = (float)normal_world[0];
      const float ny_w = (float)normal_world[1];
      const float nz_w = (float)normal_world[2];
      for (int s = -steps; s <= steps; ++s) {
        const float dist = (float)s * voxel;
        const int ix = cx_v + floor_scaled(dist * nx_w, voxel);
        const int iy = cy_v + floor_scaled(dist * ny_w, voxel);
        const int iz = cz_v + floor_scaled(dist * nz_w, voxel);
        if (!(ix >= 0 && iy >= 0 && iz >= 0 && ix < dims[0] && iy < dims[1] && iz < dims[2])) continue;
        const float wx = (float)origin[0] + ((float)ix + 0.5f) * voxel;
        const float wy = (float)origin[1] + ((float)iy + 0.5f) * voxel;
        const float wz = (float)origin[2] + ((float)iz + 0.5f) * voxel;
        const double v_w[3] = {(double)wx, (double)wy, (double)wz};
        double vc[3], v_c[3];
        mat3_vec(R_wc, v_w, vc);
        for (int i = 0; i < 3; ++i) v_c[i] = vc[i] + t_wc[i];
        if (v_c[2] <= 1e-6) continue;
        const int px_i = (int)lround(cfg->fx * v_c[0] / v_c[2] + cfg->cx);
        const int py_i = (int)lround(cfg->fy * v_c[1] / v_c[2] + cfg->cy);
        if (px_i < 0 || px_i >= width || py_i < 0 || py_i >= height) continue;
        const double diff = d_axis_m - v_c[2];
        if (fabs(diff) > (double)trunc) continue;
        const float sdf = (float)(diff / (double)trunc);
        const size_t idx = ((size_t)iz * dims[1] + iy) * dims[0] + ix;
        const float w_old = weight[idx];
        const float w_sum = w_old + w_new;
        if (w_sum > 0.0f) {
          tsdf[idx] = (w_old * tsdf[idx] + w_new * sdf) / w_sum;
          weight[idx] = w_sum;
        }
      }
      ++integrated;
    }
  }
  return integrated;
}

/* SurfaceGradient (tsdf_internal.h:154-187). */
static int surface_gradient(const int32_t dims[3], const float* tsdf, const float* weight, int ix, int iy, int iz,
                            float* onx, float* ony, float* onz) {
  static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  const size_t i0 = ((size_t)iz * dims[1] + iy) * dims[0] + ix;
  const float c = tsdf[i0], cw = weight[i0];
  if (cw <= 0.0f) return 0;
  if (c > 0.0f) return 0;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f;
  int has_positive = 0;
  for (int k = 0; k < 6; ++k) {
    const int a = ix + off[k][0], b = iy + off[k][1], cc = iz + off[k][2];
    if (!(a >= 0 && b >= 0 && cc >= 0 && a < dims[0] && b < dims[1] && cc < dims[2])) continue;
    const size_t j = ((size_t)cc * dims[1] + b) * dims[0] + a;
    if (weight[j] > 0.0f && tsdf[j] > 0.0f) {
      has_positive = 1;
      nx += (float)off[k][0];
      ny += (float)off[k][1];
      nz += (float)off[k][2];
    }
  }
  if (!has_positive) return 0;
  const float len = sqrtf(nx * nx + ny * ny + nz * nz);
  if (len < 1e-9f) return 0;
  *onx = nx / len;
  *ony = ny / len;
  *onz = nz / len;
  return 1;
}

/* TsdfVolume::ExtractPoints (tsdf_fusion.cpp:106-140): zero-crossing voxels
 * in (iz, iy, ix) order; position = voxel centre, normal = the normalised
 * sum of the unit offsets towards fused free-space neighbours, confidence =
 * min(1, weight / 64).  Returns the count; writes at most `cap` points. */
int64_t orc_tsdf_extract(const orc_tsdf_config* cfg, const float* tsdf, const float* weight, int64_t cap,
                         double* pos, double* nrm, float* conf, int64_t* voxel_index) {
  int32_t dims[3];
  orc_tsdf_dims(cfg, dims);
  const float voxel = (float)cfg->voxel_size_m;
  /* VoxelToWorld (tsdf_fusion.cpp:76-81): the FP64 origin plus the FP32
     offset, rounded to FP32 */
  const double ox = (double)(float)cfg->origin_x, oy = (double)(float)cfg->origin_y,
               oz = (double)(float)cfg->origin_z;
  int64_t n = 0;
  for (int iz = 0; iz < dims[2]; ++iz)
    for (int iy = 0; iy < dims[1]; ++iy)
      for (int ix = 0; ix < dims[0]; ++ix) {
        float nx, ny, nz;
        if (!surface_gradient(dims, tsdf, weight, ix, iy, iz, &nx, &ny, &nz)) continue;
        if (n < cap) {
          const size_t i0 = ((size_t)iz * dims[1] + iy) * dims[0] + ix;
          pos[3 * n + 0] = (double)(float)(ox + (double)(((float)ix + 0.5f) * voxel));
          pos[3 * n + 1] = (double)(float)(oy + (double)(((float)iy + 0.5f) * voxel));
          pos[3 * n + 2] = (double)(float)(oz + (double)(((float)iz + 0.5f) * voxel));
          nrm[3 * n + 0] = (double)nx;
          nrm[3 * n + 1] = (double)ny;
          nrm[3 * n + 2] = (double)nz;
          const float q = weight[i0] / 64.0f;
          conf[n] = q < 1.0f ? q : 1.0f;
          if (voxel_index) voxel_index[n] = (int64_t)i0;
        }
        ++n;
      }
  return n;
}
