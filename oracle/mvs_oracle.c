/*
 * mvs_oracle.c -- CPU restatement of the reference PatchMatch MVS path.
 *
 * TEST INFRASTRUCTURE ONLY (see mvs_oracle.h).  Compile with
 * -ffp-contract=off: the restatement keeps the reference's double-precision
 * evaluation order, and a fused multiply-add would change the last bits.
 *
 * Citations are file:line into the reference project.
 */
#define _GNU_SOURCE
#include "mvs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------ */
/* small FP64 vector helpers; each keeps the reference's summation order     */
/* (core/include/recon/linalg.h:224-232: s = 0; s += m[i][j]*v[j] for j).   */
/* ------------------------------------------------------------------------ */

static void mat_vec(const double* m, const double* v, double* out) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += m[i * 3 + j] * v[j];
    out[i] = s;
  }
}

static void mat_t_vec(const double* m, const double* v, double* out) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += m[j * 3 + i] * v[j];
    out[i] = s;
  }
}

static double vnorm3(const double* v) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s += v[i] * v[i];
  return sqrt(s);
}

/* CameraPose::CameraToWorld = R^T (p - t)   (camera.h:69-71) */
static void camera_to_world(const orc_pose* p, const double* pc, double* out) {
  double d[3];
  for (int i = 0; i < 3; ++i) d[i] = pc[i] - p->t[i];
  mat_t_vec(p->r, d, out);
}

/* CameraPose::WorldToCamera = R p + t   (camera.h:73-75) */
static void world_to_camera(const orc_pose* p, const double* pw, double* out) {
  double r[3];
  mat_vec(p->r, pw, r);
  for (int i = 0; i < 3; ++i) out[i] = r[i] + p->t[i];
}

/* CameraPose::CenterWorld = -(R^T t)   (camera.h:77) */
static void center_world(const orc_pose* p, double* out) {
  double r[3];
  mat_t_vec(p->r, p->t, r);
  for (int i = 0; i < 3; ++i) out[i] = -r[i];
}

/* ------------------------------------------------------------------------ */
/* camera model                                                              */
/* ------------------------------------------------------------------------ */

/* camera.cpp:33-45 */
void orc_apply_distortion(const orc_intrinsics* k, double x, double y, double* ox, double* oy) {
  const double r2 = x * x + y * y;
  const double r4 = r2 * r2;
  const double r6 = r4 * r2;
  const double radial = 1.0 + k->k1 * r2 + k->k2 * r4 + k->k3 * r6;
  const double pxy = k->p1 * x * y + k->p2 * (r2 + 2.0 * x * x);
  const double pxy2 = k->p1 * (r2 + 2.0 * y * y) + k->p2 * x * y;
  *ox = x * radial + pxy;
  *oy = y * radial + pxy2;
}

/* camera.cpp:47-129: damped Newton with the analytic Jacobian, <= 50 steps,
 * residual tolerance 1e-15, up to 20 step halvings. */
void orc_remove_distortion(const orc_intrinsics* k, double xd, double yd, double* ox, double* oy) {
  if (k->k1 == 0.0 && k->k2 == 0.0 && k->k3 == 0.0 && k->p1 == 0.0 && k->p2 == 0.0) {
    *ox = xd;
    *oy = yd;
    return;
  }
  double x = xd, y = yd;
  for (int iter = 0; iter < 50; ++iter) {
    double xr = 0.0, yr = 0.0;
    orc_apply_distortion(k, x, y, &xr, &yr);
    const double ex = xd - xr;
    const double ey = yd - yr;
    const double err = sqrt(ex * ex + ey * ey);
    if (err < 1e-15) break;
    const double r2 = x * x + y * y;
    const double r4 = r2 * r2;
    const double radial = 1.0 + k->k1 * r2 + k->k2 * r4 + k->k3 * r4 * r2;
    const double dr = k->k1 + 2.0 * k->k2 * r2 + 3.0 * k->k3 * r4;
    const double j00 = radial + 2.0 * x * x * dr + 2.0 * k->p1 * y + k->p2 * (3.0 * x * x + y * y);
    const double j01 = 2.0 * x * y * dr + k->p1 * (x * x + 3.0 * y * y) + 2.0 * k->p2 * x * y;
    const double j10 = 2.0 * x * y * dr + 2.0 * k->p1 * x + k->p2 * (x * x + 3.0 * y * y);
    const double j11 = radial + 2.0 * y * y * dr + k->p1 * (3.0 * x * x + y * y) + 2.0 * k->p2 * x * y;
    const double det = j00 * j11 - j01 * j10;
    if (fabs(det) < 1e-12) break;
    const double dx = (j11 * ex - j01 * ey) / det;
    const double dy = (-j10 * ex + j00 * ey) / det;
    double lambda = 1.0;
    int accepted = 0;
    for (int ls = 0; ls < 20; ++ls) {
      const double xn = x + lambda * dx;
      const double yn = y + lambda * dy;
      double xrn = 0.0, yrn = 0.0;
      orc_apply_distortion(k, xn, yn, &xrn, &yrn);
      const double rn = sqrt((xd - xrn) * (xd - xrn) + (yd - yrn) * (yd - yrn));
      if (rn < err) {
        x = xn;
        y = yn;
        accepted = 1;
        break;
      }
      lambda *= 0.5;
    }
    if (!accepted) break;
  }
  *ox = x;
  *oy = y;
}

/* camera.cpp:131-150 (PixelToNormalized + PixelToRay) */
void orc_pixel_to_ray(const orc_intrinsics* k, double u, double v, double ray[3]) {
  const double xn = (u - k->cx) / k->fx;
  const double yn = (v - k->cy) / k->fy;
  double x = 0.0, y = 0.0;
  orc_remove_distortion(k, xn, yn, &x, &y);
  ray[0] = x;
  ray[1] = y;
  ray[2] = 1.0;
}

/* camera.cpp:152-162 */
int32_t orc_project_point(const orc_intrinsics* k, const double p[3], double* u, double* v) {
  if (p[2] <= 1e-9) return 0;
  const double x = p[0] / p[2];
  const double y = p[1] / p[2];
  double xd = 0.0, yd = 0.0;
  orc_apply_distortion(k, x, y, &xd, &yd);
  *u = k->fx * xd + k->cx;
  *v = k->fy * yd + k->cy;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* NCC and candidate cost                                                    */
/* ------------------------------------------------------------------------ */

/* patchmatch_stereo.cpp:78-100.  Pixel index == coordinate (no half-pixel
 * shift); out of range when u<0, v<0, u>w-1 or v>h-1. */
int32_t orc_sample_bilinear(const uint8_t* img, int32_t w, int32_t h, double u, double v, double* out) {
  if (u < 0.0 || v < 0.0 || u > (double)(w - 1) || v > (double)(h - 1)) return 0;
  const int x0 = (int)floor(u);
  const int y0 = (int)floor(v);
  const int x1 = x0 + 1 < w - 1 ? x0 + 1 : w - 1;
  const int y1 = y0 + 1 < h - 1 ? y0 + 1 : h - 1;
  const double fx = u - x0;
  const double fy = v - y0;
  const double p00 = img[y0 * w + x0];
  const double p10 = img[y0 * w + x1];
  const double p01 = img[y1 * w + x0];
  const double p11 = img[y1 * w + x1];
  const double top = p00 * (1.0 - fx) + p10 * fx;
  const double bot = p01 * (1.0 - fx) + p11 * fx;
  *out = top * (1.0 - fy) + bot * fy;
  return 1;
}

/* Weak-texture variance floor hard-coded in the reference
 * (patchmatch_stereo.cpp:38, used at :260). */
#define ORC_WEAK_TEXTURE_VARIANCE 12.0

/* patchmatch_stereo.cpp:214-274 */
orc_ncc_result orc_compute_ncc(const uint8_t* ref, int32_t ref_w, int32_t ref_h,
                               const uint8_t* src, int32_t src_w, int32_t src_h,
                               double ref_u, double ref_v, double src_u, double src_v,
                               int32_t patch_size) {
  orc_ncc_result r;
  r.valid = 0;
  r.ncc = 0.0;
  r.weak_texture = 0;
  r.valid_samples = 0;
  const int half = patch_size / 2;
  double sum_ref = 0.0, sum_src = 0.0;
  double sum_ref2 = 0.0, sum_src2 = 0.0, sum_cross = 0.0;
  int valid = 0;
  for (int dy = -half; dy <= half; ++dy) {
    for (int dx = -half; dx <= half; ++dx) {
      double vr = 0.0, vs = 0.0;
      if (!orc_sample_bilinear(ref, ref_w, ref_h, ref_u + dx, ref_v + dy, &vr)) continue;
      if (!orc_sample_bilinear(src, src_w, src_h, src_u + dx, src_v + dy, &vs)) continue;
      sum_ref += vr;
      sum_src += vs;
      sum_ref2 += vr * vr;
      sum_src2 += vs * vs;
      sum_cross += vr * vs;
      ++valid;
    }
  }
  if (valid < patch_size * patch_size / 2) {
    r.valid = 0;
    r.ncc = 0.0;
    return r;
  }
  const double n = (double)valid;
  const double mean_ref = sum_ref / n;
  const double mean_src = sum_src / n;
  const double var_ref = sum_ref2 / n - mean_ref * mean_ref;
  const double var_src = sum_src2 / n - mean_src * mean_src;
  r.weak_texture = var_ref < ORC_WEAK_TEXTURE_VARIANCE;
  const double denom = sqrt(var_ref * var_src);
  if (denom < 1e-9) {
    r.valid = 0;
    r.ncc = 0.0;
    return r;
  }
  double ncc = (sum_cross / n - mean_ref * mean_src) / denom;
  if (ncc < -1.0) ncc = -1.0;
  if (ncc > 1.0) ncc = 1.0;
  r.ncc = ncc;
  r.valid = 1;
  r.valid_samples = valid;
  return r;
}

/* patchmatch_stereo.cpp:327-336 */
static double inverse_depth_to_depth(double inv) { return inv <= 1e-9 ? 1e9 : 1.0 / inv; }
static double depth_to_inverse_depth(double d) { return d < 1e-9 ? 1e9 : 1.0 / d; }

static int intrinsics_are_global(const orc_views* v) { return v->num_src_intr == v->num_src_poses; }

static const orc_intrinsics* src_intrinsics(const orc_views* v, int k) {
  return intrinsics_are_global(v) ? &v->src_intr[v->source_indices[k]] : &v->src_intr[k];
}

/* patchmatch_stereo.cpp:344-418 (EvaluateCandidate) */
orc_cost_result orc_evaluate_candidate(const orc_views* v, const orc_config* cfg,
                                       double u, double vv, double inv_depth) {
  orc_cost_result res;
  res.cost = 1e30;
  res.ncc_sum = 0.0;
  res.weight_sum = 0.0;
  res.weak_texture_count = 0;
  res.valid_views = 0;
  if (inv_depth <= 1e-9) return res;
  const double depth = inverse_depth_to_depth(inv_depth);
  if (depth < cfg->min_depth_m || depth > cfg->max_depth_m) return res;
  double ray[3], p_cam[3], p_world[3];
  orc_pixel_to_ray(v->ref_intr, u, vv, ray);
  for (int i = 0; i < 3; ++i) p_cam[i] = ray[i] * depth;
  camera_to_world(v->ref_pose, p_cam, p_world);
  for (int k = 0; k < v->num_src; ++k) {
    const int si = v->source_indices[k];
    const orc_pose* sp = &v->src_poses[si];
    const orc_intrinsics* si_k = src_intrinsics(v, k);
    double p_src[3];
    world_to_camera(sp, p_world, p_src);
    if (p_src[2] <= 1e-6) continue;
    double su = 0.0, sv = 0.0;
    if (!orc_project_point(si_k, p_src, &su, &sv)) continue;
    const orc_ncc_result ncc = orc_compute_ncc(v->ref, v->ref_w, v->ref_h, v->src[k], v->src_w[k],
                                               v->src_h[k], u, vv, su, sv, cfg->patch_size);
    if (!ncc.valid) continue;
    ++res.valid_views;
    if (ncc.weak_texture) ++res.weak_texture_count;
    const double weight = 1.0;
    res.ncc_sum += weight * ncc.ncc;
    res.weight_sum += weight;
  }
  if (res.weight_sum <= 0.0) return res;
  const double mean_ncc = res.ncc_sum / res.weight_sum;
  res.cost = 1.0 - mean_ncc;
  if (res.cost > 3.0 * cfg->photo_threshold) res.cost = 1e30;
  return res;
}

void orc_evaluate_candidates(const orc_views* v, const orc_config* cfg, int32_t n,
                             const int32_t* px, const int32_t* py, const double* inv,
                             double* out_cost, int32_t* out_valid_views) {
  for (int32_t i = 0; i < n; ++i) {
    const orc_cost_result c = orc_evaluate_candidate(v, cfg, px[i] + 0.5, py[i] + 0.5, inv[i]);
    out_cost[i] = c.cost;
    out_valid_views[i] = c.valid_views;
  }
}

/* ------------------------------------------------------------------------ */
/* PatchMatch (patchmatch_stereo.cpp:422-764)                                */
/* ------------------------------------------------------------------------ */

/* patchmatch_stereo.cpp:104-125: xorshift64* (12/25/27, 0x2545F4914F6CDD1D). */
typedef struct { uint64_t state; } orc_rng;
static void rng_init(orc_rng* r, uint64_t seed) { r->state = seed ? seed : 0x9E3779B97F4A7C15ull; }
uint32_t orc_xorshift_next(uint64_t* s) {
  *s ^= *s >> 12;
  *s ^= *s << 25;
  *s ^= *s >> 27;
  return (uint32_t)((*s * 0x2545F4914F6CDD1Dull) >> 32);
}
static double rng_uniform(orc_rng* r) { return (double)orc_xorshift_next(&r->state) / 4294967296.0; }
static double rng_signed(orc_rng* r) { return rng_uniform(r) * 2.0 - 1.0; }

static int hardware_threads(void) {
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

static int resolve_threads(const orc_config* cfg) {
  int t = cfg->num_threads;
  if (t <= 0) t = hardware_threads();
  return t < 1 ? 1 : t;
}

/* patchmatch_stereo.cpp:434-485 */
int32_t orc_pm_prepare(const orc_views* v, const orc_config* cfg,
                       double* inv_min, double* inv_max, double* baseline) {
  if (v->ref == NULL) return 0;
  if (v->num_src <= 0) return 0;
  const int glob = v->num_src_intr == v->num_src_poses;
  const int rel = v->num_src_intr == v->num_src;
  if (!glob && !rel) return 0;
  /* The reference range-checks source_indices only under the global form
   * (:459-466); out-of-range indices under the relative form are undefined
   * behaviour there, and rejected here. */
  for (int k = 0; k < v->num_src; ++k) {
    const int si = v->source_indices[k];
    if (si < 0 || si >= v->num_src_poses) return 0;
  }
  double rc[3];
  center_world(v->ref_pose, rc);
  double bsum = 0.0;
  for (int k = 0; k < v->num_src; ++k) {
    double sc[3], d[3];
    center_world(&v->src_poses[v->source_indices[k]], sc);
    for (int i = 0; i < 3; ++i) d[i] = sc[i] - rc[i];
    bsum += vnorm3(d);
  }
  *baseline = bsum / (double)v->num_src;
  if (*baseline < 1e-9) return 0;
  *inv_min = depth_to_inverse_depth(cfg->max_depth_m);
  *inv_max = depth_to_inverse_depth(cfg->min_depth_m);
  if (!(*inv_max > *inv_min) || *inv_min <= 0.0) return 0;
  return 1;
}

typedef struct {
  const orc_views* v;
  const orc_config* cfg;
  int block_id, block_count;
  /* init */
  const double* inv;
  double* cost;
  int32_t* support;
  /* sweep */
  int iter, dir, rows_per_block;
  double inv_min, inv_max;
  const double* snap_inv;
  const double* snap_cost;
  double* out_inv;
  double* out_cost;
  int32_t* out_support;
} orc_task;

/* patchmatch_stereo.cpp:553-567 */
static void* init_block(void* arg) {
  orc_task* t = (orc_task*)arg;
  const orc_views* v = t->v;
  const int rows = (v->ref_h + t->block_count - 1) / t->block_count;
  const int y0 = t->block_id * rows;
  const int y1 = v->ref_h < y0 + rows ? v->ref_h : y0 + rows;
  for (int y = y0; y < y1; ++y) {
    for (int x = 0; x < v->ref_w; ++x) {
      const size_t idx = (size_t)y * v->ref_w + x;
      const orc_cost_result c = orc_evaluate_candidate(v, t->cfg, x + 0.5, y + 0.5, t->inv[idx]);
      t->cost[idx] = c.cost;
      t->support[idx] = c.valid_views;
    }
  }
  return NULL;
}

static void run_blocks(orc_task* tasks, int count, void* (*fn)(void*)) {
  if (count <= 1) {
    fn(&tasks[0]);
    return;
  }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)count);
  for (int b = 0; b < count; ++b) pthread_create(&th[b], NULL, fn, &tasks[b]);
  for (int b = 0; b < count; ++b) pthread_join(th[b], NULL);
  free(th);
}

/* patchmatch_stereo.cpp:487-581 */
void orc_pm_init(const orc_views* v, const orc_config* cfg,
                 const double* seed_points, int32_t num_seeds,
                 double* inv, double* cost, int32_t* support) {
  double inv_min = 0, inv_max = 0, baseline = 0;
  if (!orc_pm_prepare(v, cfg, &inv_min, &inv_max, &baseline)) return;
  const size_t n = (size_t)v->ref_w * v->ref_h;
  uint8_t* initialized = (uint8_t*)calloc(n, 1);
  for (size_t i = 0; i < n; ++i) {
    inv[i] = 0.0;
    cost[i] = 1e30;
    support[i] = 0;
  }
  orc_rng rng;
  rng_init(&rng, 0x5DEECE66Dull);
  /* :499-533 sparse seeding on a 32-px grid: every pixel of a cell takes
   * the mean depth of the seeds that fell into it. */
  if (seed_points != NULL && num_seeds > 0) {
    const int grid = 32;
    const int gx = (v->ref_w + grid - 1) / grid;
    const int gy = (v->ref_h + grid - 1) / grid;
    double* csum = (double*)calloc((size_t)gx * gy, sizeof(double));
    int* ccount = (int*)calloc((size_t)gx * gy, sizeof(int));
    /* the reference sums each bucket in insertion order (:524-525) */
    for (int i = 0; i < num_seeds; ++i) {
      const double su = seed_points[3 * i], sv = seed_points[3 * i + 1], sd = seed_points[3 * i + 2];
      if (su < 0 || sv < 0 || su >= v->ref_w || sv >= v->ref_h) continue;
      if (sd <= 0.0) continue;
      int cx = (int)su / grid;
      int cy = (int)sv / grid;
      if (cx > gx - 1) cx = gx - 1;
      if (cy > gy - 1) cy = gy - 1;
      csum[(size_t)cy * gx + cx] += sd;
      ccount[(size_t)cy * gx + cx] += 1;
    }
    for (int y = 0; y < v->ref_h; ++y) {
      for (int x = 0; x < v->ref_w; ++x) {
        int cx = x / grid, cy = y / grid;
        if (cx > gx - 1) cx = gx - 1;
        if (cy > gy - 1) cy = gy - 1;
        const size_t c = (size_t)cy * gx + cx;
        if (ccount[c] == 0) continue;
        const double depth = csum[c] / (double)ccount[c];
        const size_t idx = (size_t)y * v->ref_w + x;
        inv[idx] = depth_to_inverse_depth(depth);
        initialized[idx] = 1;
      }
    }
    free(csum);
    free(ccount);
  }
  /* :536-539 one global generator in row-major order */
  for (size_t idx = 0; idx < n; ++idx) {
    if (initialized[idx]) continue;
    inv[idx] = inv_min + rng_uniform(&rng) * (inv_max - inv_min);
  }
  free(initialized);
  /* :543-581 initial cost over row blocks (independent of the block count) */
  const int threads = resolve_threads(cfg);
  orc_task* tasks = (orc_task*)calloc((size_t)threads, sizeof(orc_task));
  for (int b = 0; b < threads; ++b) {
    tasks[b].v = v;
    tasks[b].cfg = cfg;
    tasks[b].block_id = b;
    tasks[b].block_count = threads;
    tasks[b].inv = inv;
    tasks[b].cost = cost;
    tasks[b].support = support;
  }
  run_blocks(tasks, threads, init_block);
  free(tasks);
}

static void try_update(orc_task* t, size_t idx, double cand, const orc_cost_result* c) {
  if (c->cost < t->out_cost[idx]) {
    t->out_cost[idx] = c->cost;
    t->out_inv[idx] = cand;
    t->out_support[idx] = c->valid_views;
  }
}

/* patchmatch_stereo.cpp:642-723: one row block of one direction sweep. */
static void* sweep_block(void* arg) {
  orc_task* t = (orc_task*)arg;
  const orc_views* v = t->v;
  const orc_config* cfg = t->cfg;
  const int W = v->ref_w, H = v->ref_h;
  const int yb0 = t->block_id * t->rows_per_block;
  const int yb1 = H < yb0 + t->rows_per_block ? H : yb0 + t->rows_per_block;
  if (yb0 >= yb1) return NULL;
  orc_rng rng;
  rng_init(&rng, 0x5DEECE66Dull + (uint64_t)t->block_id * 0x9E3779B97F4A7C15ull +
                     (uint64_t)t->iter * 0xC2B2AE3D27D4EB4Full);
  const int reverse_x = (t->dir == 1 || t->dir == 3);
  const int reverse_y = (t->dir >= 2);
  const int y_start = reverse_y ? yb1 - 1 : yb0;
  const int y_end = reverse_y ? yb0 - 1 : yb1;
  const int y_step = reverse_y ? -1 : 1;
  static const int kNeighbor[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
  for (int y = y_start; y != y_end; y += y_step) {
    const int x_start = reverse_x ? W - 1 : 0;
    const int x_end = reverse_x ? -1 : W;
    const int x_step = reverse_x ? -1 : 1;
    for (int x = x_start; x != x_end; x += x_step) {
      const size_t idx = (size_t)y * W + x;
      if (cfg->propagation_enabled) {
        for (int nb = 0; nb < 4; ++nb) {
          const int nx = x + kNeighbor[nb][0];
          const int ny = y + kNeighbor[nb][1];
          if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
          const size_t nidx = (size_t)ny * W + nx;
          if (t->snap_cost[nidx] >= 1e29) continue;
          const orc_cost_result c = orc_evaluate_candidate(v, cfg, x + 0.5, y + 0.5, t->snap_inv[nidx]);
          try_update(t, idx, t->snap_inv[nidx], &c);
        }
      }
      double radius = t->out_inv[idx] * cfg->random_search_radius_ratio;
      for (int k = 0; k < cfg->random_search_count; ++k) {
        const double cand = t->out_inv[idx] + rng_signed(&rng) * radius;
        if (cand < t->inv_min || cand > t->inv_max) {
          radius *= 0.5;
          continue;
        }
        const orc_cost_result c = orc_evaluate_candidate(v, cfg, x + 0.5, y + 0.5, cand);
        try_update(t, idx, cand, &c);
        radius *= 0.5;
      }
      if (rng_uniform(&rng) < cfg->restart_ratio) {
        const double cand = t->inv_min + rng_uniform(&rng) * (t->inv_max - t->inv_min);
        const orc_cost_result c = orc_evaluate_candidate(v, cfg, x + 0.5, y + 0.5, cand);
        try_update(t, idx, cand, &c);
      }
    }
  }
  return NULL;
}

/* patchmatch_stereo.cpp:607-741 for one (iter, dir). */
void orc_pm_sweep(const orc_views* v, const orc_config* cfg, int32_t iter, int32_t dir,
                  const double* inv, const double* cost, const int32_t* support,
                  double* out_inv, double* out_cost, int32_t* out_support) {
  double inv_min = 0, inv_max = 0, baseline = 0;
  if (!orc_pm_prepare(v, cfg, &inv_min, &inv_max, &baseline)) return;
  const size_t n = (size_t)v->ref_w * v->ref_h;
  memcpy(out_inv, inv, n * sizeof(double));
  memcpy(out_cost, cost, n * sizeof(double));
  memcpy(out_support, support, n * sizeof(int32_t));
  const int threads = resolve_threads(cfg);
  const int hb = v->ref_h / 16 > 1 ? v->ref_h / 16 : 1;
  const int block_count = threads < hb ? threads : hb;
  const int rows_per_block = (v->ref_h + block_count - 1) / block_count;
  orc_task* tasks = (orc_task*)calloc((size_t)block_count, sizeof(orc_task));
  for (int b = 0; b < block_count; ++b) {
    orc_task* t = &tasks[b];
    t->v = v;
    t->cfg = cfg;
    t->block_id = b;
    t->block_count = block_count;
    t->iter = iter;
    t->dir = dir;
    t->rows_per_block = rows_per_block;
    t->inv_min = inv_min;
    t->inv_max = inv_max;
    t->snap_inv = inv;
    t->snap_cost = cost;
    t->out_inv = out_inv;
    t->out_cost = out_cost;
    t->out_support = out_support;
  }
  run_blocks(tasks, block_count, sweep_block);
  free(tasks);
}

/* patchmatch_stereo.cpp:744-763 */
uint32_t orc_pm_output(const orc_views* v, const orc_config* cfg,
                       const double* inv, const double* cost, const int32_t* support,
                       float* depth, uint8_t* support_count, float* confidence) {
  const size_t n = (size_t)v->ref_w * v->ref_h;
  for (size_t i = 0; i < n; ++i) {
    depth[i] = nanf("");
    support_count[i] = 0;
    confidence[i] = 0.0f;
  }
  uint32_t filled = 0;
  for (size_t idx = 0; idx < n; ++idx) {
    if (cost[idx] >= 1e29) continue;
    const double d = inverse_depth_to_depth(inv[idx]);
    if (d < cfg->min_depth_m || d > cfg->max_depth_m) continue;
    depth[idx] = (float)d;
    support_count[idx] = (uint8_t)(support[idx] < 255 ? support[idx] : 255);
    double pc = cost[idx];
    if (pc < 0.0) pc = 0.0;
    if (pc > 1.0) pc = 1.0;
    confidence[idx] = (float)(1.0 - pc);
    ++filled;
  }
  return filled;
}

uint32_t orc_patchmatch_stereo(const orc_views* v, const orc_config* cfg,
                               const double* seed_points, int32_t num_seeds,
                               float* depth, uint8_t* support_count, float* confidence) {
  if (v->ref == NULL || depth == NULL) return 0;
  double inv_min = 0, inv_max = 0, baseline = 0;
  if (!orc_pm_prepare(v, cfg, &inv_min, &inv_max, &baseline)) return 0;
  const size_t n = (size_t)v->ref_w * v->ref_h;
  double* inv = (double*)malloc(n * sizeof(double));
  double* cost = (double*)malloc(n * sizeof(double));
  int32_t* sup = (int32_t*)malloc(n * sizeof(int32_t));
  double* inv2 = (double*)malloc(n * sizeof(double));
  double* cost2 = (double*)malloc(n * sizeof(double));
  int32_t* sup2 = (int32_t*)malloc(n * sizeof(int32_t));
  orc_pm_init(v, cfg, seed_points, num_seeds, inv, cost, sup);
  const int dirs = cfg->propagation_directions > 1 ? cfg->propagation_directions : 1;
  for (int iter = 0; iter < cfg->iterations; ++iter) {
    for (int dir = 0; dir < dirs; ++dir) {
      orc_pm_sweep(v, cfg, iter, dir, inv, cost, sup, inv2, cost2, sup2);
      double* ti = inv; inv = inv2; inv2 = ti;
      double* tc = cost; cost = cost2; cost2 = tc;
      int32_t* ts = sup; sup = sup2; sup2 = ts;
    }
  }
  const uint32_t filled = orc_pm_output(v, cfg, inv, cost, sup, depth, support_count, confidence);
  free(inv); free(cost); free(sup); free(inv2); free(cost2); free(sup2);
  return filled;
}

/* ------------------------------------------------------------------------ */
/* RefineSubpixel (patchmatch_stereo.cpp:770-979)                            */
/* ------------------------------------------------------------------------ */

/* patchmatch_stereo.cpp:42-75: Gauss-Jordan with partial pivoting. */
static int solve_linear_3x3(const double A[3][3], const double b[3], double x[3]) {
  double m[3][4];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) m[i][j] = A[i][j];
    m[i][3] = b[i];
  }
  for (int col = 0; col < 3; ++col) {
    int pivot = col;
    for (int r = col + 1; r < 3; ++r)
      if (fabs(m[r][col]) > fabs(m[pivot][col])) pivot = r;
    if (fabs(m[pivot][col]) < 1e-18) return 0;
    if (pivot != col) {
      for (int j = 0; j < 4; ++j) {
        const double tmp = m[col][j];
        m[col][j] = m[pivot][j];
        m[pivot][j] = tmp;
      }
    }
    for (int r = 0; r < 3; ++r) {
      if (r == col) continue;
      const double factor = m[r][col] / m[col][col];
      for (int j = col; j < 4; ++j) m[r][j] -= factor * m[col][j];
    }
  }
  for (int i = 0; i < 3; ++i) {
    if (fabs(m[i][i]) < 1e-18) return 0;
    x[i] = m[i][3] / m[i][i];
  }
  return 1;
}

static double refine_eval(const orc_views* v, const orc_config* cfg, double u, double vv, double inv) {
  return orc_evaluate_candidate(v, cfg, u, vv, inv).cost;
}

/* The per-pixel body of RefineSubpixel (:817-976).  Returns 1 when the
 * reference would write the pixel. */
static int refine_one(const orc_views* v, const orc_config* cfg, double inv_min, double inv_max,
                      double inv_per_px, int x, int y, float d0, double* best_inv, double* best_cost) {
  if (!isfinite(d0)) return 0;
  const double u = x + 0.5;
  const double vv = y + 0.5;
  const double inv0 = depth_to_inverse_depth(d0);
  if (inv0 < inv_min || inv0 > inv_max) return 0;
  const int fit_points = cfg->subpixel_fit_points > 3 ? cfg->subpixel_fit_points : 3;
  const int half_fit = fit_points / 2;
  const double fit_step = inv_per_px * 0.5;
  double fit_cost[64];
  int fit_ok = fit_points <= 64;
  for (int k = 0; k < fit_points && fit_ok; ++k) fit_cost[k] = 1e30;
  for (int k = 0; k < fit_points && k < 64; ++k) {
    const double d = inv0 + (k - half_fit) * fit_step;
    if (d < inv_min || d > inv_max) {
      fit_ok = 0;
      break;
    }
    fit_cost[k] = refine_eval(v, cfg, u, vv, d);
    if (fit_cost[k] >= 1e29) fit_ok = 0;
  }
  double best_d = inv0;
  double best_c = refine_eval(v, cfg, u, vv, inv0);
  if (fit_ok) {
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, t0 = 0, t1 = 0, t2 = 0;
    for (int k = 0; k < fit_points; ++k) {
      const double xx = (double)(k - half_fit);
      const double c = fit_cost[k];
      s0 += 1.0;
      s1 += xx;
      s2 += xx * xx;
      s3 += xx * xx * xx;
      s4 += xx * xx * xx * xx;
      t0 += c;
      t1 += xx * c;
      t2 += xx * xx * c;
    }
    const double A[3][3] = {{s4, s3, s2}, {s3, s2, s1}, {s2, s1, s0}};
    const double b[3] = {t2, t1, t0};
    double sol[3] = {0.0, 0.0, 0.0};
    if (solve_linear_3x3(A, b, sol)) {
      const double a = sol[0];
      const double bb = sol[1];
      if (fabs(a) > 1e-12) {
        const double vertex = -bb / (2.0 * a);
        /* :896-899 the vertex, in sample-index units, is added to the
         * inverse depth without the fit_step scale (kept as is). */
        if (vertex >= -(double)half_fit && vertex <= (double)half_fit) {
          const double cand = inv0 + vertex;
          const double cc = refine_eval(v, cfg, u, vv, cand);
          if (cc < best_c) {
            best_c = cc;
            best_d = cand;
          }
        }
      }
    }
  }
  {
    double lo = best_d - inv_per_px * 1.0;
    double hi = best_d + inv_per_px * 1.0;
    if (lo < inv_min) lo = inv_min;
    if (hi > inv_max) hi = inv_max;
    if (hi > lo) {
      const double inv_phi = 0.6180339887498949;
      double c1 = hi - inv_phi * (hi - lo);
      double c2 = lo + inv_phi * (hi - lo);
      double f1 = refine_eval(v, cfg, u, vv, c1);
      double f2 = refine_eval(v, cfg, u, vv, c2);
      for (int k = 0; k < cfg->subpixel_iterations; ++k) {
        if (f1 < f2) {
          hi = c2;
          c2 = c1;
          f2 = f1;
          c1 = hi - inv_phi * (hi - lo);
          f1 = refine_eval(v, cfg, u, vv, c1);
        } else {
          lo = c1;
          c1 = c2;
          f1 = f2;
          c2 = lo + inv_phi * (hi - lo);
          f2 = refine_eval(v, cfg, u, vv, c2);
        }
      }
      const double cand_mid = 0.5 * (lo + hi);
      const double cc_mid = refine_eval(v, cfg, u, vv, cand_mid);
      if (cc_mid < best_c) {
        best_c = cc_mid;
        best_d = cand_mid;
      }
      if (f1 < best_c) {
        best_c = f1;
        best_d = c1;
      }
      if (f2 < best_c) {
        best_c = f2;
        best_d = c2;
      }
    }
  }
  *best_inv = best_d;
  *best_cost = best_c;
  if (best_d < inv_min || best_d > inv_max) return 0;
  const double final_depth = inverse_depth_to_depth(best_d);
  if (final_depth < cfg->min_depth_m || final_depth > cfg->max_depth_m) return 0;
  return 1;
}

static int refine_prepare(const orc_views* v, const orc_config* cfg, double* inv_min,
                          double* inv_max, double* inv_per_px) {
  if (v->ref == NULL) return 0;
  if (v->num_src <= 0) return 0;
  for (int k = 0; k < v->num_src; ++k) {
    const int si = v->source_indices[k];
    if (si < 0 || si >= v->num_src_poses) return 0;
  }
  double rc[3];
  center_world(v->ref_pose, rc);
  double bsum = 0.0;
  for (int k = 0; k < v->num_src; ++k) {
    double sc[3], d[3];
    center_world(&v->src_poses[v->source_indices[k]], sc);
    for (int i = 0; i < 3; ++i) d[i] = sc[i] - rc[i];
    bsum += vnorm3(d);
  }
  const double baseline = bsum / (double)v->num_src;
  if (baseline < 1e-9) return 0;
  *inv_min = depth_to_inverse_depth(cfg->max_depth_m);
  *inv_max = depth_to_inverse_depth(cfg->min_depth_m);
  const double focal_px = 0.5 * (v->ref_intr->fx + v->ref_intr->fy);
  const int glob = v->num_src_intr == v->num_src_poses;
  const int rel = v->num_src_intr == v->num_src;
  if (!glob && !rel) return 0;
  *inv_per_px = 1.0 / (focal_px * baseline);
  return 1;
}

uint32_t orc_refine_subpixel(const orc_views* v, const orc_config* cfg,
                             float* depth, uint8_t* support_count, float* confidence) {
  (void)support_count;
  if (depth == NULL) return 0;
  double inv_min, inv_max, inv_per_px;
  if (!refine_prepare(v, cfg, &inv_min, &inv_max, &inv_per_px)) return 0;
  uint32_t refined = 0;
  for (int y = 0; y < v->ref_h; ++y) {
    for (int x = 0; x < v->ref_w; ++x) {
      const size_t idx = (size_t)y * v->ref_w + x;
      double bi = 0, bc = 0;
      if (!refine_one(v, cfg, inv_min, inv_max, inv_per_px, x, y, depth[idx], &bi, &bc)) continue;
      depth[idx] = (float)inverse_depth_to_depth(bi);
      double pc = bc;
      if (pc < 0.0) pc = 0.0;
      if (pc > 1.0) pc = 1.0;
      confidence[idx] = (float)(1.0 - pc);
      ++refined;
    }
  }
  return refined;
}

void orc_refine_pixels(const orc_views* v, const orc_config* cfg, const float* depth,
                       int32_t n, const int32_t* px, const int32_t* py,
                       double* out_best_inv, double* out_best_cost, int32_t* out_written) {
  double inv_min, inv_max, inv_per_px;
  const int ok = refine_prepare(v, cfg, &inv_min, &inv_max, &inv_per_px);
  for (int32_t i = 0; i < n; ++i) {
    out_best_inv[i] = NAN;
    out_best_cost[i] = 1e30;
    out_written[i] = 0;
    if (!ok) continue;
    const size_t idx = (size_t)py[i] * v->ref_w + px[i];
    out_written[i] = refine_one(v, cfg, inv_min, inv_max, inv_per_px, px[i], py[i], depth[idx],
                                &out_best_inv[i], &out_best_cost[i]);
  }
}

/* ------------------------------------------------------------------------ */
/* FuseDepthMaps (patchmatch_stereo.cpp:985-1089)                            */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t key;
  double sum_pos[3];
  double sum_normal[3];
  double sum_conf;
  uint32_t count;
  int used;
} orc_voxel;

typedef struct {
  orc_voxel* slots;
  size_t cap;
  size_t size;
} orc_voxel_map;

static uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

static orc_voxel* voxel_find(orc_voxel_map* m, int64_t key) {
  if ((m->size + 1) * 2 > m->cap) {
    const size_t ncap = m->cap ? m->cap * 2 : 1024;
    orc_voxel* ns = (orc_voxel*)calloc(ncap, sizeof(orc_voxel));
    for (size_t i = 0; i < m->cap; ++i) {
      if (!m->slots[i].used) continue;
      size_t h = mix64((uint64_t)m->slots[i].key) & (ncap - 1);
      while (ns[h].used) h = (h + 1) & (ncap - 1);
      ns[h] = m->slots[i];
    }
    free(m->slots);
    m->slots = ns;
    m->cap = ncap;
  }
  size_t h = mix64((uint64_t)key) & (m->cap - 1);
  while (m->slots[h].used && m->slots[h].key != key) h = (h + 1) & (m->cap - 1);
  if (!m->slots[h].used) {
    memset(&m->slots[h], 0, sizeof(orc_voxel));
    m->slots[h].used = 1;
    m->slots[h].key = key;
    ++m->size;
  }
  return &m->slots[h];
}

static int cmp_voxel_key(const void* a, const void* b) {
  const orc_voxel* va = *(const orc_voxel* const*)a;
  const orc_voxel* vb = *(const orc_voxel* const*)b;
  return va->key < vb->key ? -1 : (va->key > vb->key ? 1 : 0);
}

int64_t orc_fuse_depth_maps(const orc_depth_map* maps, int32_t num_maps,
                            const orc_pose* poses, const orc_intrinsics* intr,
                            const orc_config* cfg, int64_t max_out,
                            int64_t* out_keys, double* out_pos, double* out_normal,
                            float* out_conf, uint32_t* out_count) {
  if (num_maps <= 0) return 0;
  const double voxel = cfg->fusion_voxel_size_m;
  if (voxel <= 0.0) return 0;
  orc_voxel_map vm = {NULL, 0, 0};
  for (int mi = 0; mi < num_maps; ++mi) {
    const orc_depth_map* dm = &maps[mi];
    if (dm->depth == NULL) continue;
    const orc_pose* pose = &poses[mi];
    const orc_intrinsics* k = &intr[mi];
    for (int y = 0; y < dm->height; ++y) {
      for (int x = 0; x < dm->width; ++x) {
        const size_t idx = (size_t)y * dm->width + x;
        const float depth = dm->depth[idx];
        if (!isfinite(depth)) continue;
        if (dm->support_count[idx] < cfg->min_view_consistency) continue;
        if (cfg->photo_threshold < 1.0) {
          const float photo_cost = 1.0f - dm->confidence[idx];
          if (photo_cost > cfg->photo_threshold) continue;
        }
        double ray[3], p_cam[3], p_world[3], nr[3], nw[3];
        orc_pixel_to_ray(k, x + 0.5, y + 0.5, ray);
        for (int i = 0; i < 3; ++i) p_cam[i] = ray[i] * (double)depth;
        camera_to_world(pose, p_cam, p_world);
        /* normal = -(R^T ray).normalized()  (:1038) */
        mat_t_vec(pose->r, ray, nr);
        const double nn = vnorm3(nr);
        if (nn < 1e-15) {
          nw[0] = nw[1] = nw[2] = 0.0;
        } else {
          for (int i = 0; i < 3; ++i) nw[i] = nr[i] / nn;
        }
        for (int i = 0; i < 3; ++i) nw[i] = -nw[i];
        const int64_t vx = (int64_t)floor(p_world[0] / voxel);
        const int64_t vy = (int64_t)floor(p_world[1] / voxel);
        const int64_t vz = (int64_t)floor(p_world[2] / voxel);
        /* :1045-1046 XOR-mixed key; distinct voxels with one key merge. */
        const int64_t key = (int64_t)(((uint64_t)vx * 73856093ull) ^ ((uint64_t)vy * 19349663ull) ^
                                      ((uint64_t)vz * 83492791ull));
        orc_voxel* acc = voxel_find(&vm, key);
        for (int i = 0; i < 3; ++i) acc->sum_pos[i] += p_world[i];
        for (int i = 0; i < 3; ++i) acc->sum_normal[i] += nw[i];
        acc->sum_conf += dm->confidence[idx];
        ++acc->count;
      }
    }
  }
  const int64_t total = (int64_t)vm.size;
  if (out_keys != NULL && total > 0) {
    orc_voxel** list = (orc_voxel**)malloc(sizeof(orc_voxel*) * vm.size);
    size_t j = 0;
    for (size_t i = 0; i < vm.cap; ++i)
      if (vm.slots[i].used) list[j++] = &vm.slots[i];
    qsort(list, vm.size, sizeof(orc_voxel*), cmp_voxel_key);
    for (size_t i = 0; i < vm.size && (int64_t)i < max_out; ++i) {
      const orc_voxel* a = list[i];
      const double cnt = (double)a->count;
      double pos[3], nrm[3];
      for (int q = 0; q < 3; ++q) pos[q] = a->sum_pos[q] / cnt;
      for (int q = 0; q < 3; ++q) nrm[q] = a->sum_normal[q];
      const double n = vnorm3(nrm);
      if (n > 1e-12) {
        /* Vec::normalize (linalg.h:77-81) */
        const double n2 = vnorm3(nrm);
        if (!(n2 < 1e-15))
          for (int q = 0; q < 3; ++q) nrm[q] /= n2;
      } else {
        nrm[0] = 0.0;
        nrm[1] = 0.0;
        nrm[2] = 1.0;
      }
      const double ce = (a->sum_conf / cnt) * sqrt(cnt);
      out_keys[i] = a->key;
      for (int q = 0; q < 3; ++q) out_pos[3 * i + q] = pos[q];
      for (int q = 0; q < 3; ++q) out_normal[3 * i + q] = nrm[q];
      out_conf[i] = (float)(ce < 1.0 ? ce : 1.0);
      out_count[i] = a->count;
    }
    free(list);
  }
  free(vm.slots);
  return total;
}

/* ------------------------------------------------------------------------ */
/* SelectSourceViews (patchmatch_stereo.cpp:133-211)                         */
/* ------------------------------------------------------------------------ */

typedef struct {
  int index;
  double score;
} orc_candidate;

int32_t orc_select_source_views(const orc_pose* ref_pose, const orc_pose* poses,
                                int32_t num_poses, const orc_intrinsics* intr,
                                const orc_config* cfg, int32_t* out_indices) {
  (void)intr;
  const double kPi = 3.14159265358979323846;
  orc_candidate* c = (orc_candidate*)malloc(sizeof(orc_candidate) * (size_t)(num_poses > 0 ? num_poses : 1));
  int nc = 0;
  double rc[3];
  center_world(ref_pose, rc);
  for (int i = 0; i < num_poses; ++i) {
    if (i == cfg->ref_view_index) continue;
    double sc[3], base[3];
    center_world(&poses[i], sc);
    for (int q = 0; q < 3; ++q) base[q] = sc[q] - rc[q];
    if (vnorm3(base) < 1e-6) continue;
    const double z_ref = cfg->reference_depth_m;
    const double z_src = z_ref + base[2];
    if (z_src <= 1e-6) continue;
    const double scale_ratio = z_ref / z_src;
    if (fabs(scale_ratio - 1.0) > cfg->max_view_scale_mismatch) continue;
    double rel_world[3], rel_cam[3];
    for (int q = 0; q < 3; ++q) rel_world[q] = sc[q] - rc[q];
    mat_vec(ref_pose->r, rel_world, rel_cam);
    const double dist = vnorm3(rel_cam);
    if (dist < 1e-6) continue;
    double cz = rel_cam[2] / dist;
    if (cz < -1.0) cz = -1.0;
    if (cz > 1.0) cz = 1.0;
    const double angle_deg = acos(cz) * 180.0 / kPi;
    double angle_score;
    if (angle_deg < cfg->ideal_angle_min_deg) {
      angle_score = angle_deg / cfg->ideal_angle_min_deg;
    } else if (angle_deg > cfg->ideal_angle_max_deg) {
      const double s = 1.0 - (angle_deg - cfg->ideal_angle_max_deg) / (cfg->ideal_angle_max_deg * 2.0);
      angle_score = s > 0.0 ? s : 0.0;
    } else {
      angle_score = 1.0;
    }
    c[nc].index = i;
    c[nc].score = angle_score * cfg->view_angle_weight;
    ++nc;
  }
  /* Descending by score.  The reference calls std::sort; for <= 16
   * candidates libstdc++ runs a plain insertion sort there, which keeps
   * equal scores in input order -- the stable insertion sort below
   * reproduces that.  Beyond 16 candidates with tied scores the reference
   * order is implementation-defined. */
  for (int i = 1; i < nc; ++i) {
    const orc_candidate val = c[i];
    int j = i;
    while (j > 0 && val.score > c[j - 1].score) {
      c[j] = c[j - 1];
      --j;
    }
    c[j] = val;
  }
  int out = 0;
  for (int i = 0; i < nc && out < cfg->num_views; ++i) out_indices[out++] = c[i].index;
  free(c);
  return out;
}

/* ------------------------------------------------------------------------ */
/* Plane-induced homography cost (no reference CPU counterpart)              */
/* ------------------------------------------------------------------------ */

/* Pixel-centre bilinear read: coordinate c covers index c - 0.5; the
 * in-range rule of SampleBilinear applies to the index coordinate. */
static int sample_centre(const uint8_t* img, int w, int h, double cu, double cv, double* out) {
  return orc_sample_bilinear(img, w, h, cu - 0.5, cv - 0.5, out);
}

/* SampleBilinear's rules (index == coordinate) on an FP32 image. */
static int sample_bilinear_f(const float* img, int w, int h, double u, double v, double* out) {
  if (u < 0.0 || v < 0.0 || u > (double)(w - 1) || v > (double)(h - 1)) return 0;
  const int x0 = (int)floor(u), y0 = (int)floor(v);
  const int x1 = x0 + 1 < w ? x0 + 1 : w - 1, y1 = y0 + 1 < h ? y0 + 1 : h - 1;
  const double fx = u - x0, fy = v - y0;
  const double top = img[(size_t)y0 * w + x0] * (1.0 - fx) + img[(size_t)y0 * w + x1] * fx;
  const double bot = img[(size_t)y1 * w + x0] * (1.0 - fx) + img[(size_t)y1 * w + x1] * fx;
  *out = top * (1.0 - fy) + bot * fy;
  return 1;
}

/* Source sample k at (u, v): 8-bit or FP32 image, pixel-centre or the
 * reference's index == coordinate convention. */
static int sample_source(const orc_views* v, int k, double u, double vv, int half_pixel, double* out) {
  if (v->src_f != NULL) {
    const double o = half_pixel ? 0.0 : 0.5;
    return sample_bilinear_f(v->src_f[k], v->src_w[k], v->src_h[k], u - o, vv - o, out);
  }
  if (half_pixel) return orc_sample_bilinear(v->src[k], v->src_w[k], v->src_h[k], u, vv, out);
  return sample_centre(v->src[k], v->src_w[k], v->src_h[k], u, vv, out);
}

/* The plane cost with an optional bar: a caller that keeps the hypothesis
 * only if its cost is below `beat` may stop once the views evaluated so far
 * bound the final cost above it -- view costs lie in [0, 2], so with K views
 * averaged (best_k, or all), n valid so far and r views left the final cost
 * is at least (sum of the min(K, n + r) - r lowest costs so far) /
 * min(K, n + r).  A stopped evaluation returns cost 1e30 (rejected, as the
 * full one would be); beat >= 1e299 evaluates every view. */
static orc_plane_result plane_cost_core(const orc_views* v, const orc_config* cfg, int32_t best_k,
                                        int32_t x, int32_t y, double inv_depth, const double n[3],
                                        int32_t half_pixel, double beat) {
  orc_plane_result res;
  memset(&res, 0, sizeof(res));
  res.cost = 1e30;
  for (int k = 0; k < 32; ++k) res.view_cost[k] = 1e30;
  if (inv_depth <= 1e-9) return res;
  const double depth = 1.0 / inv_depth;
  if (depth < cfg->min_depth_m || depth > cfg->max_depth_m) return res;
  const orc_intrinsics* kr = v->ref_intr;
  const double uc = x + 0.5, vc = y + 0.5;
  const double r0[3] = {(uc - kr->cx) / kr->fx, (vc - kr->cy) / kr->fy, 1.0};
  const double X0[3] = {r0[0] * depth, r0[1] * depth, depth};
  const double delta = n[0] * X0[0] + n[1] * X0[1] + n[2] * X0[2];
  if (!(delta < 0.0)) return res; /* plane must face the camera */
  /* grazing planes (normal within ~3 degrees of perpendicular to the ray)
     are not plane-mode hypotheses */
  if (!(n[0] * r0[0] + n[1] * r0[1] + n[2] < -0.05 * sqrt(r0[0] * r0[0] + r0[1] * r0[1] + 1.0))) return res;
  const int half = cfg->patch_size / 2;
  const int min_valid = cfg->patch_size * cfg->patch_size / 2;
  double refc[3];
  center_world(v->ref_pose, refc);
  int nvalid = 0;
  double vcost[32];
  const int nsrc = v->num_src < 32 ? v->num_src : 32;
  for (int k = 0; k < nsrc; ++k) {
    if (beat < 1e299 && nvalid > 0) {
      const int left = nsrc - k;
      const int K = best_k > 0 ? best_k : nsrc;
      const int kk = K < nvalid + left ? K : nvalid + left;
      const int j = kk - left;
      if (j > 0) {
        double low[32];
        for (int i = 0; i < nvalid; ++i) { /* the costs so far, ascending */
          int q = i;
          while (q > 0 && low[q - 1] > vcost[i]) {
            low[q] = low[q - 1];
            --q;
          }
          low[q] = vcost[i];
        }
        double lb = 0.0;
        for (int i = 0; i < j; ++i) lb += low[i];
        if (lb > beat * (1.0 + 1e-12) * kk) {
          res.cost = 1e30;
          res.valid_views = 0;
          return res;
        }
      }
    }
    const orc_pose* sp = &v->src_poses[v->source_indices[k]];
    const orc_intrinsics* ks = src_intrinsics(v, k);
    /* A = R_s R_r^T, b = t_s - A t_r: reference-camera point -> source camera */
    double A[9], b[3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int q = 0; q < 3; ++q) s += sp->r[i * 3 + q] * v->ref_pose->r[j * 3 + q];
        A[i * 3 + j] = s;
      }
    double At[3];
    mat_vec(A, v->ref_pose->t, At);
    for (int i = 0; i < 3; ++i) b[i] = sp->t[i] - At[i];
    /* centre point must lie in front of the source camera */
    double Xs0[3];
    mat_vec(A, X0, Xs0);
    for (int i = 0; i < 3; ++i) Xs0[i] += b[i];
    if (Xs0[2] <= 1e-6) continue;
    double sr = 0, ss = 0, srr = 0, sss = 0, srs = 0;
    double edge = 1e30;
    int valid = 0;
    for (int dy = -half; dy <= half; ++dy) {
      for (int dx = -half; dx <= half; ++dx) {
        const int rx = x + dx, ry = y + dy;
        double vr = 0.0;
        if (half_pixel) {
          if (v->ref_f != NULL) {
            if (!sample_bilinear_f(v->ref_f, v->ref_w, v->ref_h, rx + 0.5, ry + 0.5, &vr)) continue;
          } else if (!orc_sample_bilinear(v->ref, v->ref_w, v->ref_h, rx + 0.5, ry + 0.5, &vr)) {
            continue;
          }
        } else {
          if (rx < 0 || ry < 0 || rx > v->ref_w - 1 || ry > v->ref_h - 1) continue;
          vr = v->ref_f != NULL ? (double)v->ref_f[(size_t)ry * v->ref_w + rx] : v->ref[(size_t)ry * v->ref_w + rx];
        }
        const double rp[3] = {(rx + 0.5 - kr->cx) / kr->fx, (ry + 0.5 - kr->cy) / kr->fy, 1.0};
        const double nd = n[0] * rp[0] + n[1] * rp[1] + n[2] * rp[2];
        if (!(nd < 0.0)) continue;
        const double lam = delta / nd;
        const double X[3] = {rp[0] * lam, rp[1] * lam, rp[2] * lam};
        double Xs[3];
        mat_vec(A, X, Xs);
        for (int i = 0; i < 3; ++i) Xs[i] += b[i];
        if (Xs[2] <= 1e-9) continue;
        const double su = ks->fx * (Xs[0] / Xs[2]) + ks->cx;
        const double sv = ks->fy * (Xs[1] / Xs[2]) + ks->cy;
        double vs = 0.0;
        if (!sample_source(v, k, su, sv, half_pixel, &vs)) continue;
        {
          const double o = half_pixel ? 0.0 : 0.5;
          const double fu = (su - o) - floor(su - o), fv = (sv - o) - floor(sv - o);
          double e = fu < 1.0 - fu ? fu : 1.0 - fu;
          if (fv < e) e = fv;
          if (1.0 - fv < e) e = 1.0 - fv;
          if (e < edge) edge = e;
        }
        sr += vr;
        ss += vs;
        srr += vr * vr;
        sss += vs * vs;
        srs += vr * vs;
        ++valid;
      }
    }
    if (valid < min_valid) continue;
    const double nn = (double)valid;
    const double mr = sr / nn, ms = ss / nn;
    const double var_r = srr / nn - mr * mr;
    const double var_s = sss / nn - ms * ms;
    const double denom = sqrt(var_r * var_s);
    if (denom < 1e-9) continue;
    double ncc = (srs / nn - mr * ms) / denom;
    if (ncc < -1.0) ncc = -1.0;
    if (ncc > 1.0) ncc = 1.0;
    res.view_cost[k] = 1.0 - ncc;
    res.view_valid[k] = 1;
    res.view_edge[k] = edge;
    vcost[nvalid++] = 1.0 - ncc;
  }
  res.valid_views = nvalid;
  if (nvalid == 0) return res;
  /* mean of the best_k lowest view costs */
  for (int i = 1; i < nvalid; ++i) {
    const double t = vcost[i];
    int j = i;
    while (j > 0 && vcost[j - 1] > t) {
      vcost[j] = vcost[j - 1];
      --j;
    }
    vcost[j] = t;
  }
  const int kk = best_k > 0 && best_k < nvalid ? best_k : nvalid;
  double s = 0.0;
  for (int i = 0; i < kk; ++i) s += vcost[i];
  res.cost = s / kk;
  if (res.cost > 3.0 * cfg->photo_threshold) res.cost = 1e30;
  return res;
}

orc_plane_result orc_plane_cost(const orc_views* v, const orc_config* cfg, int32_t best_k,
                                int32_t x, int32_t y, double inv_depth, const double n[3],
                                int32_t half_pixel) {
  return plane_cost_core(v, cfg, best_k, x, y, inv_depth, n, half_pixel, 1e300);
}

typedef struct {
  const orc_views* v;
  const orc_config* cfg;
  int32_t best_k, i0, i1, half_pixel;
  const int32_t *px, *py;
  const double *inv, *normals;
  double* out_cost;
  int32_t* out_valid_views;
  double* out_view_cost;
} plane_costs_task;

static void* plane_costs_run(void* arg) {
  const plane_costs_task* T = (const plane_costs_task*)arg;
  for (int32_t i = T->i0; i < T->i1; ++i) {
    const orc_plane_result r =
        orc_plane_cost(T->v, T->cfg, T->best_k, T->px[i], T->py[i], T->inv[i], &T->normals[3 * i], T->half_pixel);
    T->out_cost[i] = r.cost;
    T->out_valid_views[i] = r.valid_views;
    if (T->out_view_cost)
      for (int k = 0; k < T->v->num_src; ++k) T->out_view_cost[(size_t)i * T->v->num_src + k] = r.view_cost[k];
  }
  return NULL;
}

/* Independent hypotheses: split over cfg->num_threads threads (0 = all). */
void orc_plane_costs(const orc_views* v, const orc_config* cfg, int32_t best_k, int32_t n,
                     const int32_t* px, const int32_t* py, const double* inv,
                     const double* normals, double* out_cost, int32_t* out_valid_views,
                     double* out_view_cost, int32_t half_pixel) {
  int threads = cfg->num_threads > 0 ? cfg->num_threads : (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (threads < 1) threads = 1;
  if (threads > n / 64 + 1) threads = n / 64 + 1;
  plane_costs_task* tasks = (plane_costs_task*)malloc(sizeof(plane_costs_task) * (size_t)threads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
  for (int t = 0; t < threads; ++t) {
    plane_costs_task T = {v, cfg, best_k, (int32_t)((long long)n * t / threads),
                          (int32_t)((long long)n * (t + 1) / threads), half_pixel, px, py, inv, normals,
                          out_cost, out_valid_views, out_view_cost};
    tasks[t] = T;
    pthread_create(&th[t], NULL, plane_costs_run, &tasks[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
  free(th);
  free(tasks);
}

void orc_plane_edge_distance(const orc_views* v, const orc_config* cfg, int32_t best_k, int32_t n,
                             const int32_t* px, const int32_t* py, const double* inv,
                             const double* normals, double* out_dist) {
  const int nsrc = v->num_src < 32 ? v->num_src : 32;
  for (int32_t h = 0; h < n; ++h) {
    const orc_plane_result r =
        plane_cost_core(v, cfg, best_k, px[h], py[h], inv[h], &normals[3 * h], 0, 1e300);
    /* the views the cost averages: the best_k lowest view costs */
    int order[32], m = 0;
    for (int k = 0; k < nsrc; ++k) {
      if (!r.view_valid[k]) continue;
      int q = m++;
      while (q > 0 && r.view_cost[order[q - 1]] > r.view_cost[k]) {
        order[q] = order[q - 1];
        --q;
      }
      order[q] = k;
    }
    const int kk = best_k > 0 && best_k < m ? best_k : m;
    double d = 1e30;
    for (int i = 0; i < kk; ++i)
      if (r.view_edge[order[i]] < d) d = r.view_edge[order[i]];
    out_dist[h] = d;
  }
}

/* ------------------------------------------------------------------------ */
/* Geometric consistency (no reference CPU counterpart)                      */
/* ------------------------------------------------------------------------ */

void orc_relative_transform_f32(const orc_pose* ref, const orc_pose* src, float Af[9], float bf[3]) {
  double A[9], At[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int q = 0; q < 3; ++q) s += src->r[i * 3 + q] * ref->r[j * 3 + q];
      A[i * 3 + j] = s;
    }
  mat_vec(A, ref->t, At);
  for (int i = 0; i < 9; ++i) Af[i] = (float)A[i];
  for (int i = 0; i < 3; ++i) bf[i] = (float)(src->t[i] - At[i]);
}

/* One (ref pixel, source map) test.  The operation order here is the
 * contract the GPU kernel follows. */
static int consistent_one(const float* A, const float* b, const float* Ai, const float* bi,
                          float fxr, float fyr, float cxr, float cyr,
                          float fxs, float fys, float cxs, float cys,
                          const float* dsrc, int ws, int hs, int x, int y, float z,
                          float rel_max, float reproj2_max) {
  const float xr = ((float)x + 0.5f - cxr) / fxr;
  const float yr = ((float)y + 0.5f - cyr) / fyr;
  const float P0 = xr * z, P1 = yr * z, P2 = z;
  const float Q0 = A[0] * P0 + A[1] * P1 + A[2] * P2 + b[0];
  const float Q1 = A[3] * P0 + A[4] * P1 + A[5] * P2 + b[1];
  const float Q2 = A[6] * P0 + A[7] * P1 + A[8] * P2 + b[2];
  if (!(Q2 > 1e-6f)) return 0;
  const float us = fxs * (Q0 / Q2) + cxs;
  const float vs = fys * (Q1 / Q2) + cys;
  if (!(us >= 0.0f && us < (float)ws && vs >= 0.0f && vs < (float)hs)) return 0;
  const int ix = (int)us, iy = (int)vs;
  const float zs = dsrc[(size_t)iy * ws + ix];
  if (!(zs > 0.0f) || !isfinite(zs)) return 0;
  const float xs = ((float)ix + 0.5f - cxs) / fxs;
  const float ys = ((float)iy + 0.5f - cys) / fys;
  const float S0 = xs * zs, S1 = ys * zs, S2 = zs;
  const float B0 = Ai[0] * S0 + Ai[1] * S1 + Ai[2] * S2 + bi[0];
  const float B1 = Ai[3] * S0 + Ai[4] * S1 + Ai[5] * S2 + bi[1];
  const float B2 = Ai[6] * S0 + Ai[7] * S1 + Ai[8] * S2 + bi[2];
  if (!(B2 > 1e-6f)) return 0;
  const float rel = fabsf(B2 - z) / z;
  const float ur = fxr * (B0 / B2) + cxr;
  const float vr = fyr * (B1 / B2) + cyr;
  const float du = ur - ((float)x + 0.5f);
  const float dv = vr - ((float)y + 0.5f);
  const float e2 = du * du + dv * dv;
  return rel <= rel_max && e2 <= reproj2_max;
}

void orc_geo_consistency(const orc_depth_map* maps, int32_t num_maps,
                         const orc_pose* poses, const orc_intrinsics* intr,
                         int32_t r, const orc_consistency_params* p,
                         uint8_t* out_count, uint8_t* out_keep) {
  const orc_depth_map* dr = &maps[r];
  const size_t n = (size_t)dr->width * dr->height;
  const float reproj2 = p->reproj_px_max * p->reproj_px_max;
  float (*A)[9] = malloc(sizeof(float[9]) * (size_t)num_maps);
  float (*b)[3] = malloc(sizeof(float[3]) * (size_t)num_maps);
  float (*Ai)[9] = malloc(sizeof(float[9]) * (size_t)num_maps);
  float (*bi)[3] = malloc(sizeof(float[3]) * (size_t)num_maps);
  for (int s = 0; s < num_maps; ++s) {
    orc_relative_transform_f32(&poses[r], &poses[s], A[s], b[s]);
    orc_relative_transform_f32(&poses[s], &poses[r], Ai[s], bi[s]);
  }
  const float fxr = (float)intr[r].fx, fyr = (float)intr[r].fy, cxr = (float)intr[r].cx, cyr = (float)intr[r].cy;
  for (size_t idx = 0; idx < n; ++idx) {
    const int x = (int)(idx % (size_t)dr->width), y = (int)(idx / (size_t)dr->width);
    const float z = dr->depth[idx];
    int count = 0;
    if (z > 0.0f && isfinite(z)) {
      for (int s = 0; s < num_maps; ++s) {
        if (s == r || maps[s].depth == NULL) continue;
        count += consistent_one(A[s], b[s], Ai[s], bi[s], fxr, fyr, cxr, cyr,
                                (float)intr[s].fx, (float)intr[s].fy, (float)intr[s].cx, (float)intr[s].cy,
                                maps[s].depth, maps[s].width, maps[s].height, x, y, z,
                                p->rel_depth_max, reproj2);
      }
    }
    out_count[idx] = (uint8_t)(count < 255 ? count : 255);
    out_keep[idx] = (uint8_t)(count >= p->min_views && z > 0.0f && isfinite(z));
  }
  free(A);
  free(b);
  free(Ai);
  free(bi);
}

/* ------------------------------------------------------------------------ */
/* Undistortion remap (no reference CPU counterpart)                         */
/* ------------------------------------------------------------------------ */

void orc_undistort(const uint8_t* img, int32_t w, int32_t h, const orc_intrinsics* k, float* out) {
  for (int j = 0; j < h; ++j) {
    for (int i = 0; i < w; ++i) {
      const double xn = (i + 0.5 - k->cx) / k->fx;
      const double yn = (j + 0.5 - k->cy) / k->fy;
      double xd = 0.0, yd = 0.0;
      orc_apply_distortion(k, xn, yn, &xd, &yd);
      const double ud = k->fx * xd + k->cx;
      const double vd = k->fy * yd + k->cy;
      double val = 0.0;
      if (!sample_centre(img, w, h, ud, vd, &val)) val = 0.0;
      out[(size_t)j * w + i] = (float)val;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Plane-mode PatchMatch in FP64 (no reference counterpart)                  */
/* ------------------------------------------------------------------------ */
/* The GPU engine's plane-mode search restated with every cost evaluated in
 * FP64 by orc_plane_cost (pixel-centre windows): the same red-black
 * schedule, the same 8 adaptive propagation regions and 5 refinement
 * hypotheses per half-sweep, the same counter-based random streams
 * (splitmix64 finaliser), and the same golden-section refinement.  Random
 * unit vectors use cos / sin in FP64 where the GPU uses its FP32 intrinsics,
 * so the two runs draw the same hypotheses up to ~1e-6 in the normals.  It is
 * the FP64 run the mixed-precision forms are measured against. */

static uint64_t pm_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
typedef struct {
  uint64_t s;
} pm_rng;
static float pm_uniform(pm_rng* g) {
  g->s = pm_mix64(g->s);
  return (float)(uint32_t)(g->s >> 40) * (1.0f / 16777216.0f);
}
static float pm_sym(pm_rng* g) { return pm_uniform(g) * 2.0f - 1.0f; }
static pm_rng pm_pixel_rng(uint64_t seed, int idx, int iter, int salt) {
  pm_rng g;
  g.s = pm_mix64(seed ^ ((uint64_t)idx * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)(iter + 1) << 40) ^
                 ((uint64_t)salt << 56));
  return g;
}

static void pm_random_normal(pm_rng* g, double rx, double ry, double n[3]) {
  const double rn = 1.0 / sqrt(rx * rx + ry * ry + 1.0);
  for (int t = 0; t < 8; ++t) {
    const double z = pm_sym(g);
    const double phi = 6.28318530718 * pm_uniform(g);
    const double r = sqrt(fmax(0.0, 1.0 - z * z));
    double a = r * cos(phi), b = r * sin(phi), c = z;
    double d = (a * rx + b * ry + c) * rn;
    if (d > 0.0) {
      a = -a;
      b = -b;
      c = -c;
      d = -d;
    }
    if (d < -0.2) {
      n[0] = a;
      n[1] = b;
      n[2] = c;
      return;
    }
  }
  n[0] = 0.0;
  n[1] = 0.0;
  n[2] = -1.0;
}

static void pm_perturb_normal(pm_rng* g, double rx, double ry, double scale, double n[3]) {
  double a = n[0] + scale * pm_sym(g), b = n[1] + scale * pm_sym(g), c = n[2] + scale * pm_sym(g);
  const double inv = 1.0 / sqrt(a * a + b * b + c * c);
  a *= inv;
  b *= inv;
  c *= inv;
  const double rn = 1.0 / sqrt(rx * rx + ry * ry + 1.0);
  if ((a * rx + b * ry + c) * rn < -0.2) {
    n[0] = a;
    n[1] = b;
    n[2] = c;
  }
}

typedef struct {
  const orc_views* v;
  const orc_config* cfg;
  int best_k;
  uint64_t seed;
  double rho_min, rho_max, inv_per_px;
  double* hyp; /* rho, nx, ny, nz per pixel */
  double* cost;
  int32_t* support;
  int stage; /* 0 init, 1 sweep, 2 refine */
  int color, iter;
  int prune; /* 1: the engine's exact shortcuts (stop a hopeless candidate, skip a repeated one) */
  int explore_iters; /* the engine's exploration schedule: 0 = the random and fronto-parallel candidates in
                        every iteration; n > 0 = in iterations < n only (drawn either way) */
  int y0, y1;
} pm_task;

/* The cost of a hypothesis; a sweep candidate passes the pixel's cost as
 * `beat` (kept only if below it), everything else 1e300. */
static double pm_eval(const pm_task* T, int x, int y, double rho, const double n[3], int32_t* support,
                      double beat) {
  *support = 0;
  if (!(rho > 0.0) || rho < T->rho_min || rho > T->rho_max) return 1e30;
  const orc_plane_result r = plane_cost_core(T->v, T->cfg, T->best_k, x, y, rho, n, 0, T->prune ? beat : 1e300);
  *support = r.valid_views;
  return r.cost;
}

static const signed char pm_near[4][7][2] = {
    {{0, -1}, {-1, -2}, {1, -2}, {-2, -3}, {2, -3}, {-3, -4}, {3, -4}},
    {{0, 1}, {-1, 2}, {1, 2}, {-2, 3}, {2, 3}, {-3, 4}, {3, 4}},
    {{-1, 0}, {-2, -1}, {-2, 1}, {-3, -2}, {-3, 2}, {-4, -3}, {-4, 3}},
    {{1, 0}, {2, -1}, {2, 1}, {3, -2}, {3, 2}, {4, -3}, {4, 3}}};

static void pm_pixel(const pm_task* T, int x, int y) {
  const orc_views* v = T->v;
  const orc_intrinsics* k = v->ref_intr;
  const int W = v->ref_w, H = v->ref_h;
  const int idx = y * W + x;
  const double rx = (x + 0.5 - k->cx) / k->fx, ry = (y + 0.5 - k->cy) / k->fy;
  double* h = T->hyp + 4 * (size_t)idx;
  if (T->stage == 0) {
    pm_rng g = pm_pixel_rng(T->seed, idx, -1, 1);
    const double rho = T->rho_min + (T->rho_max - T->rho_min) * pm_uniform(&g);
    double n[3];
    pm_random_normal(&g, rx, ry, n);
    int32_t sup;
    T->cost[idx] = pm_eval(T, x, y, rho, n, &sup, 1e300);
    T->support[idx] = sup;
    h[0] = rho;
    h[1] = n[0];
    h[2] = n[1];
    h[3] = n[2];
    return;
  }
  if (T->stage == 1) {
    double cur[4] = {h[0], h[1], h[2], h[3]};
    double cur_cost = T->cost[idx];
    int32_t cur_sup = T->support[idx];
    double last[4] = {-1.0, 0.0, 0.0, 0.0};
    for (int r = 0; r < 8; ++r) {
      int best_n = -1;
      double best_c = 1e30;
      const int cnt = r < 4 ? 7 : 11;
      for (int q = 0; q < cnt; ++q) {
        int nx_, ny_;
        if (r < 4) {
          nx_ = x + pm_near[r][q][0];
          ny_ = y + pm_near[r][q][1];
        } else {
          const int d = r - 4, off = 3 + 2 * q;
          const int sx = d == 2 ? -1 : (d == 3 ? 1 : 0), sy = d == 0 ? -1 : (d == 1 ? 1 : 0);
          nx_ = x + sx * off;
          ny_ = y + sy * off;
        }
        if (nx_ < 0 || ny_ < 0 || nx_ >= W || ny_ >= H) continue;
        const double c = T->cost[ny_ * W + nx_];
        if (c < best_c) {
          best_c = c;
          best_n = ny_ * W + nx_;
        }
      }
      if (best_n < 0 || best_c >= 1e30) continue;
      const double* hn = T->hyp + 4 * (size_t)best_n;
      const int nxp = best_n % W, nyp = best_n / W;
      const double rxn = (nxp + 0.5 - k->cx) / k->fx, ryn = (nyp + 0.5 - k->cy) / k->fy;
      const double kn = hn[1] * rxn + hn[2] * ryn + hn[3];
      const double kp = hn[1] * rx + hn[2] * ry + hn[3];
      const double rho = (kn < 0.0 && kp < 0.0) ? hn[0] * kp / kn : -1.0;
      if (!(rho > 0.0)) continue;
      /* the current plane again: same normal, inverse depth within 4e-6 relative */
      if (hn[1] == cur[1] && hn[2] == cur[2] && hn[3] == cur[3] && fabs(rho - cur[0]) <= 4e-6 * cur[0]) continue;
      /* the candidate just rejected again (its cost cannot have fallen) */
      if (T->prune && hn[1] == last[1] && hn[2] == last[2] && hn[3] == last[3] && rho == last[0]) continue;
      last[0] = rho;
      last[1] = hn[1];
      last[2] = hn[2];
      last[3] = hn[3];
      const double n[3] = {hn[1], hn[2], hn[3]};
      int32_t sup;
      const double c = pm_eval(T, x, y, rho, n, &sup, cur_cost);
      if (c < cur_cost) {
        cur_cost = c;
        cur[0] = rho;
        cur[1] = hn[1];
        cur[2] = hn[2];
        cur[3] = hn[3];
        cur_sup = sup;
      }
    }
    pm_rng g = pm_pixel_rng(T->seed, idx, T->iter, 2 + T->color);
    const double scale = ldexp(1.0, -T->iter);
    const double span = T->rho_max - T->rho_min;
    for (int q = 0; q < 5; ++q) {
      double rho = cur[0], n[3] = {cur[1], cur[2], cur[3]};
      if (q == 0) {
        rho = T->rho_min + span * pm_uniform(&g);
        pm_random_normal(&g, rx, ry, n);
      } else if (q == 4) {
        if (n[0] == 0.0 && n[1] == 0.0) continue;
        n[0] = 0.0;
        n[1] = 0.0;
        n[2] = -1.0;
      } else {
        if (q & 1) rho = cur[0] + 0.25 * span * scale * pm_sym(&g);
        if (q & 2) pm_perturb_normal(&g, rx, ry, 0.5 * scale, n);
      }
      if ((q == 0 || q == 4) && T->explore_iters > 0 && T->iter >= T->explore_iters) continue;
      int32_t sup;
      const double c = pm_eval(T, x, y, rho, n, &sup, cur_cost);
      if (c < cur_cost) {
        cur_cost = c;
        cur[0] = rho;
        cur[1] = n[0];
        cur[2] = n[1];
        cur[3] = n[2];
        cur_sup = sup;
      }
    }
    for (int i = 0; i < 4; ++i) h[i] = cur[i];
    T->cost[idx] = cur_cost;
    T->support[idx] = cur_sup;
    return;
  }
  /* stage 2: golden-section refinement of the inverse depth along the normal */
  const double c0 = T->cost[idx];
  if (!(c0 < 1e29)) return;
  const double n[3] = {h[1], h[2], h[3]};
  double best_d = h[0], best_c = c0;
  int32_t best_s = T->support[idx];
  double lo = fmax(T->rho_min, best_d - T->inv_per_px);
  double hi = fmin(T->rho_max, best_d + T->inv_per_px);
  if (hi > lo) {
    const double inv_phi = 0.618033988749895;
    double c1 = hi - inv_phi * (hi - lo), c2 = lo + inv_phi * (hi - lo);
    int32_t s1, s2, sm;
    double f1 = pm_eval(T, x, y, c1, n, &s1, 1e300), f2 = pm_eval(T, x, y, c2, n, &s2, 1e300);
    for (int q = 0; q < T->cfg->subpixel_iterations; ++q) {
      if (f1 < f2) {
        hi = c2;
        c2 = c1;
        f2 = f1;
        s2 = s1;
        c1 = hi - inv_phi * (hi - lo);
        f1 = pm_eval(T, x, y, c1, n, &s1, 1e300);
      } else {
        lo = c1;
        c1 = c2;
        f1 = f2;
        s1 = s2;
        c2 = lo + inv_phi * (hi - lo);
        f2 = pm_eval(T, x, y, c2, n, &s2, 1e300);
      }
    }
    const double mid = 0.5 * (lo + hi);
    const double fm = pm_eval(T, x, y, mid, n, &sm, 1e300);
    if (fm < best_c) {
      best_c = fm;
      best_d = mid;
      best_s = sm;
    }
    if (f1 < best_c) {
      best_c = f1;
      best_d = c1;
      best_s = s1;
    }
    if (f2 < best_c) {
      best_c = f2;
      best_d = c2;
      best_s = s2;
    }
  }
  h[0] = best_d;
  T->cost[idx] = best_c;
  T->support[idx] = best_s;
}

static void* pm_task_run(void* arg) {
  const pm_task* T = (const pm_task*)arg;
  const int W = T->v->ref_w;
  for (int y = T->y0; y < T->y1; ++y)
    for (int x = 0; x < W; ++x) {
      if (T->stage == 1 && ((x + y) & 1) != T->color) continue;
      pm_pixel(T, x, y);
    }
  return NULL;
}

static void pm_run_stage(const pm_task* base, int threads) {
  const int H = base->v->ref_h;
  const int count = threads < H ? threads : H;
  pm_task* tasks = (pm_task*)malloc(sizeof(pm_task) * (size_t)count);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)count);
  for (int b = 0; b < count; ++b) {
    tasks[b] = *base;
    tasks[b].y0 = (int)((long long)H * b / count);
    tasks[b].y1 = (int)((long long)H * (b + 1) / count);
    pthread_create(&th[b], NULL, pm_task_run, &tasks[b]);
  }
  for (int b = 0; b < count; ++b) pthread_join(th[b], NULL);
  free(th);
  free(tasks);
}

uint32_t orc_plane_patchmatch(const orc_views* v, const orc_config* cfg, int32_t best_k, uint64_t seed,
                              int32_t refine, float* depth, float* normal, float* cost_out) {
  return orc_plane_patchmatch_ex(v, cfg, best_k, seed, refine, 0, depth, normal, cost_out);
}

uint32_t orc_plane_patchmatch_ex(const orc_views* v, const orc_config* cfg, int32_t best_k, uint64_t seed,
                                 int32_t refine, int32_t prune, float* depth, float* normal, float* cost_out) {
  return orc_plane_patchmatch_ex2(v, cfg, best_k, seed, refine, prune, 0, depth, normal, cost_out);
}

uint32_t orc_plane_patchmatch_ex2(const orc_views* v, const orc_config* cfg, int32_t best_k, uint64_t seed,
                                  int32_t refine, int32_t prune, int32_t explore_iters, float* depth, float* normal,
                                  float* cost_out) {
  const size_t n = (size_t)v->ref_w * v->ref_h;
  for (size_t i = 0; i < n; ++i) {
    depth[i] = NAN;
    if (normal) normal[3 * i] = normal[3 * i + 1] = normal[3 * i + 2] = 0.0f;
    if (cost_out) cost_out[i] = 1e30f;
  }
  double inv_min, inv_max, baseline;
  if (!orc_pm_prepare(v, cfg, &inv_min, &inv_max, &baseline)) return 0;
  const orc_intrinsics* k = v->ref_intr;
  pm_task T;
  memset(&T, 0, sizeof(T));
  T.v = v;
  T.cfg = cfg;
  T.best_k = best_k;
  T.seed = seed;
  T.prune = prune != 0;
  T.explore_iters = explore_iters;
  T.rho_min = inv_min;
  T.rho_max = inv_max;
  T.inv_per_px = 1.0 / (0.5 * (k->fx + k->fy) * baseline);
  T.hyp = (double*)malloc(sizeof(double) * 4 * n);
  T.cost = (double*)malloc(sizeof(double) * n);
  T.support = (int32_t*)malloc(sizeof(int32_t) * n);
  int threads = cfg->num_threads;
  if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (threads <= 0) threads = 1;
  T.stage = 0;
  pm_run_stage(&T, threads);
  for (int it = 0; it < cfg->iterations; ++it)
    for (int c = 0; c < 2; ++c) {
      T.stage = 1;
      T.iter = it;
      T.color = c;
      pm_run_stage(&T, threads);
    }
  if (refine && cfg->subpixel_iterations > 0) {
    T.stage = 2;
    pm_run_stage(&T, threads);
  }
  uint32_t filled = 0;
  for (size_t i = 0; i < n; ++i) {
    const double rho = T.hyp[4 * i];
    if (T.cost[i] < 1e29 && rho > 0.0) {
      const double d = 1.0 / rho;
      if (d >= cfg->min_depth_m && d <= cfg->max_depth_m) {
        depth[i] = (float)d;
        ++filled;
      }
    }
    if (normal)
      for (int c = 0; c < 3; ++c) normal[3 * i + c] = (float)T.hyp[4 * i + 1 + c];
    if (cost_out) cost_out[i] = (float)T.cost[i];
  }
  free(T.hyp);
  free(T.cost);
  free(T.support);
  return filled;
}

/* ------------------------------------------------------------------------ */
/* BgraToGray (core/src/orchestrator/orchestrator.cpp:53-67)                */
/* ------------------------------------------------------------------------ */
void orc_bgra_to_gray(const uint8_t* bgra, int32_t w, int32_t h, int32_t stride, uint8_t* out) {
  for (int y = 0; y < h; ++y) {
    const uint8_t* row = bgra + (size_t)y * stride;
    for (int x = 0; x < w; ++x) {
      const int b = row[x * 4 + 0], g = row[x * 4 + 1], r = row[x * 4 + 2];
      out[(size_t)y * w + x] = (uint8_t)((77 * r + 150 * g + 29 * b) >> 8);
    }
  }
}
