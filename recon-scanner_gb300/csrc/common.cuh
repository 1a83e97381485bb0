// common.cuh -- device-side types and helpers shared by the MVS kernels.
//
// Layout in HBM (one reference view = one "job"):
//   * source images: 2-D texture objects over cudaArrays (block-linear,
//     clamp addressing, point sampling) holding (I - 128) as FP32 or FP16.
//     A bilinear sample is one tex2Dgather of the 2x2 footprint; the shift
//     by 128 keeps NCC moment sums small so that FP32 accumulation keeps
//     its precision.  8-bit inputs are exact in both formats.
//   * reference image: (I - 128) as float, row-major, plus (compat mode)
//     its 2x2 box-filtered copy, which is what the reference samples at the
//     half-pixel window positions (patchmatch_stereo.cpp:230-233).
//   * per-pixel state: plane mode float4 {inverse depth, nx, ny, nz} + float
//     cost + uint8 support; compat mode double inverse depth (the reference
//     searches in FP64) + float cost + int32 support.
//
// GB300 has ~1/60 of its FP32 rate in FP64, so window centres -- which must
// be accurate to ~1e-6 px at coordinates ~2000 px -- are computed in
// float-float arithmetic (two FP32 words, ~44-bit mantissa) from per-pixel
// rays that are formed once in FP64.  All per-sample work is FP32.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rmvs {

constexpr int kMaxSources = 32;
constexpr int kMaxBestK = 8;  // views averaged per hypothesis, at most
constexpr float kCostInf = 1e30f;

// ---------------------------------------------------------------------------
// float-float arithmetic (Dekker / Knuth error-free transformations)
// ---------------------------------------------------------------------------
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(float a) { return {a, 0.0f}; }

__device__ __forceinline__ ff ff_from_double(double d) {
  const float hi = __double2float_rn(d);
  return {hi, __double2float_rn(d - (double)hi)};
}

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  const float t = __fadd_rn(__fadd_rn(a.lo, b.lo), s.lo);
  return fast_two_sum(s.hi, t);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}

// a + b * c with b ff, c float
__device__ __forceinline__ ff ff_fma_f(ff a, ff b, float c) { return ff_add(a, ff_mul_f(b, c)); }

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// a / b: an approximate quotient, then the exactly computed remainder
// corrects it (the final error is second order in the approximation).
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float rb = rcp_approx(b.hi);
  const float q1 = a.hi * rb;
  // r = a - q1 * b
  const ff qb = ff_mul_f(b, q1);
  const ff r = ff_add(a, ff{-qb.hi, -qb.lo});
  const float q2 = r.hi * rb;
  return fast_two_sum(q1, q2);
}

// floor of an ff value and the FP32 fraction in [0, 1]
__device__ __forceinline__ void ff_floor_frac(ff a, int* i, float* frac) {
  float f = floorf(a.hi);
  float r = __fadd_rn(__fsub_rn(a.hi, f), a.lo);  // exact: a.hi - f is exact
  if (r < 0.0f) {
    f -= 1.0f;
    r += 1.0f;
  } else if (r >= 1.0f) {
    f += 1.0f;
    r -= 1.0f;
  }
  *i = (int)f;
  *frac = r;
}

// ---------------------------------------------------------------------------
// counter-based RNG (splitmix64 finaliser): deterministic, order-free
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s;
  __device__ __forceinline__ float uniform() {  // [0, 1)
    s = mix64(s);
    return (float)(uint32_t)(s >> 40) * (1.0f / 16777216.0f);
  }
  __device__ __forceinline__ float sym() { return uniform() * 2.0f - 1.0f; }
};

// ---------------------------------------------------------------------------
// view tables
// ---------------------------------------------------------------------------

// One source view of one job.  A, b map reference-camera points to this
// camera: X_s = A X_r + b (composed in FP64 on the host).
struct SrcView {
  cudaTextureObject_t tex;      // (I - 128), FP32 or FP16, clamp, point filter (gather)
  cudaTextureObject_t tex_lin;  // the same array with hardware bilinear filtering
  int w, h;
  float fx, fy, cx, cy;
  ff ffx, ffy, fcx, fcy;
  float k1, k2, k3, p1, p2;
  int distorted;
  float Ac0[3];  // A[:,0] / fx_ref
  float Ac1[3];  // A[:,1] / fy_ref
  float b[3];
  ff bff[3];
  double A[9];
  double bd[3];
  ff Aff[9];  // A in float-float (per-pixel source rays without FP64)
  // optional: a 2-D TMA map (global memory) over the texel-pair image of this
  // view -- element (x, y) = {T(x, y), T(x + 1, y)} as two FP32 words, T the
  // texels the gather object returns -- read in boxes of kStageW x kStageH
  // elements by the staged-window sweep; null when not built
  const void* pair_map;
};

// The source box one warp of the staged-window sweep holds in shared memory:
// kStageW texel pairs (8 bytes each, an even count: 16-byte TMA rows) x
// kStageH rows.  A warp's 32 pixels span 16 columns x 4 rows; with an 11 x 11
// window their footprint at unit scale is 27 x 15 texels, and the box leaves
// room for the spread of their hypotheses.
constexpr int kStageW = 40, kStageH = 24;
constexpr int kStageBytes = kStageW * kStageH * 8;

// Columns of one reference-tile plane staged by a sweep block: the tile's 32
// same-colour column pairs, 8 margin on the left and 16 on the right (a TMA
// box row of 224 bytes).  The row pitch of 56 words puts the 4 rows x 8
// consecutive pairs that one warp reads into 32 distinct banks.
constexpr int kTileCols = 56;

// Source read modes of the plane-mode kernels (Job::src_mode).
constexpr int kSrcExact = 0, kSrcTex = 1, kSrcBf16 = 2;

// One reference view: its image, camera and search state.
struct Job {
  int w, h, num_src;
  int patch_half;
  int min_valid;  // patch_size * patch_size / 2 (patchmatch_stereo.cpp:245)
  float rfx, rfy, rcx, rcy;
  double drfx, drfy, drcx, drcy;
  ff ffrx, ffry, ffrcx, ffrcy;  // the same in float-float
  int ref_distorted;
  double rk1, rk2, rk3, rp1, rp2;
  const float* ref;      // (I - 128), row-major w x h
  const float* ref_box;  // compat: 2x2 box average of (I - 128), (w-1) x (h-1) used
  const float* ref_de;   // plane mode: even / odd column planes of pref, [2][h][ref_pitch], ref_half_w used
  int ref_half_w;
  int ref_pitch;         // row pitch of ref_de in floats: ref_half_w rounded up to 4 (16-byte rows for TMA)
  // plane mode sampling convention: 0 = pixel centres (reference window =
  // pixels, source index = coordinate - 0.5); 1 = the reference's own
  // (window at x + 0.5 + dx with index == coordinate, i.e. the 2x2 box image,
  // source index == coordinate)
  int half_pixel;
  // plane mode source reads: 0 = exact FP32 bilinear from a 2x2 gather of an
  // FP32 / FP16 texture; 1 = the texture unit's bilinear filter (8-bit
  // fixed-point weights); 2 = exact FP32 bilinear from a 2x2 gather of BF16
  // bits held in a 16-bit unsigned texture
  int src_mode;
  const float* pref;     // the plane-mode reference window image: ref or ref_box
  const SrcView* src;    // num_src entries (device memory)
  // plane-mode state
  float4* hyp;   // {rho, nx, ny, nz}
  float* cost;
  uint8_t* support;
  // compat-mode state (double inverse depth as in the reference)
  double* inv;
  int32_t* isupport;
  // search range
  float rho_min, rho_max;  // inverse depth bounds
  double dinv_min, dinv_max;
  double min_depth, max_depth;
  float photo_threshold;
  int best_k;
  int prune;  // 1 = the sweep skips work that cannot change a pixel's fate (repeated candidates, hopeless windows)
  uint64_t seed;
  unsigned long long* eval_counter;  // optional: [0] hypotheses evaluated, [1] source windows sampled
  // plane-mode run parameters (read by the batched kernels per work item)
  const float* seed_depth;  // optional per-32-px-cell seed depth, seed_gx cells per row
  int seed_gx;
  int iterations;           // red-black iterations of this job
  int refine_iters;         // refinement steps; 0 = no refinement
  int refine_mode;          // 1 = golden-section on the inverse depth, 2 = Gauss-Newton on (d, theta, phi)
  float inv_per_px;         // refinement half-range: 1 px of disparity in inverse depth
  float* out_depth;
  uint8_t* out_support;
  float* out_conf;
  float* out_normal;        // optional
  float* out_cost;          // optional
  unsigned int* out_filled; // zeroed by the init kernel, counted by the output kernel
  // coarse-to-fine initialisation (optional): the plane state of this view's
  // half-resolution search; pixel (x, y) starts from the plane of its parent
  // (x / 2, y / 2), carried to its own ray
  const float4* coarse_hyp;
  const float* coarse_cost;
  int coarse_w, coarse_h;
  float crfx, crfy, crcx, crcy;  // the half-resolution reference intrinsics
  int iter_offset;               // iterations run at the coarse level: the schedule continues from there
  // exploration schedule: sweeps of iteration >= explore_iters (counted over
  // the whole schedule) evaluate no exploration candidate (the uniformly
  // random plane, the current depth on a fronto-parallel plane); 0 = every
  // iteration does
  int explore_iters;
};

// Per-pixel ray of the reference camera, FP64: pinhole fast path, or the
// damped-Newton undistortion of camera.cpp:47-129 in the reference's order.
__device__ inline void apply_distortion_d(double k1, double k2, double k3, double p1, double p2, double x,
                                          double y, double* ox, double* oy) {
  const double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
  const double r4 = __dmul_rn(r2, r2);
  const double r6 = __dmul_rn(r4, r2);
  const double radial =
      __dadd_rn(__dadd_rn(__dadd_rn(1.0, __dmul_rn(k1, r2)), __dmul_rn(k2, r4)), __dmul_rn(k3, r6));
  const double pxy = __dadd_rn(__dmul_rn(__dmul_rn(p1, x), y),
                               __dmul_rn(p2, __dadd_rn(r2, __dmul_rn(__dmul_rn(2.0, x), x))));
  const double pxy2 = __dadd_rn(__dmul_rn(p1, __dadd_rn(r2, __dmul_rn(__dmul_rn(2.0, y), y))),
                                __dmul_rn(__dmul_rn(p2, x), y));
  *ox = __dadd_rn(__dmul_rn(x, radial), pxy);
  *oy = __dadd_rn(__dmul_rn(y, radial), pxy2);
}

__device__ inline void remove_distortion_d(double k1, double k2, double k3, double p1, double p2, double xd,
                                           double yd, double* ox, double* oy) {
  if (k1 == 0.0 && k2 == 0.0 && k3 == 0.0 && p1 == 0.0 && p2 == 0.0) {
    *ox = xd;
    *oy = yd;
    return;
  }
  double x = xd, y = yd;
  for (int iter = 0; iter < 50; ++iter) {
    double xr, yr;
    apply_distortion_d(k1, k2, k3, p1, p2, x, y, &xr, &yr);
    const double ex = __dsub_rn(xd, xr);
    const double ey = __dsub_rn(yd, yr);
    const double err = __dsqrt_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
    if (err < 1e-15) break;
    const double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    const double r4 = __dmul_rn(r2, r2);
    const double radial = __dadd_rn(__dadd_rn(__dadd_rn(1.0, __dmul_rn(k1, r2)), __dmul_rn(k2, r4)),
                                    __dmul_rn(__dmul_rn(k3, r4), r2));
    const double dr = __dadd_rn(__dadd_rn(k1, __dmul_rn(__dmul_rn(2.0, k2), r2)), __dmul_rn(__dmul_rn(3.0, k3), r4));
    const double j00 = __dadd_rn(
        __dadd_rn(__dadd_rn(radial, __dmul_rn(__dmul_rn(__dmul_rn(2.0, x), x), dr)), __dmul_rn(__dmul_rn(2.0, p1), y)),
        __dmul_rn(p2, __dadd_rn(__dmul_rn(__dmul_rn(3.0, x), x), __dmul_rn(y, y))));
    const double j01 = __dadd_rn(
        __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, x), y), dr), __dmul_rn(p1, __dadd_rn(__dmul_rn(x, x), __dmul_rn(__dmul_rn(3.0, y), y)))),
        __dmul_rn(__dmul_rn(__dmul_rn(2.0, p2), x), y));
    const double j10 = __dadd_rn(
        __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, x), y), dr), __dmul_rn(__dmul_rn(2.0, p1), x)),
        __dmul_rn(p2, __dadd_rn(__dmul_rn(x, x), __dmul_rn(__dmul_rn(3.0, y), y))));
    const double j11 = __dadd_rn(
        __dadd_rn(__dadd_rn(radial, __dmul_rn(__dmul_rn(__dmul_rn(2.0, y), y), dr)),
                  __dmul_rn(p1, __dadd_rn(__dmul_rn(__dmul_rn(3.0, x), x), __dmul_rn(y, y)))),
        __dmul_rn(__dmul_rn(__dmul_rn(2.0, p2), x), y));
    const double det = __dsub_rn(__dmul_rn(j00, j11), __dmul_rn(j01, j10));
    if (fabs(det) < 1e-12) break;
    const double dx = __ddiv_rn(__dsub_rn(__dmul_rn(j11, ex), __dmul_rn(j01, ey)), det);
    const double dy = __ddiv_rn(__dadd_rn(__dmul_rn(-j10, ex), __dmul_rn(j00, ey)), det);
    double lambda = 1.0;
    bool accepted = false;
    for (int ls = 0; ls < 20; ++ls) {
      const double xn = __dadd_rn(x, __dmul_rn(lambda, dx));
      const double yn = __dadd_rn(y, __dmul_rn(lambda, dy));
      double xrn, yrn;
      apply_distortion_d(k1, k2, k3, p1, p2, xn, yn, &xrn, &yrn);
      const double a = __dsub_rn(xd, xrn), b = __dsub_rn(yd, yrn);
      const double rn = __dsqrt_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)));
      if (rn < err) {
        x = xn;
        y = yn;
        accepted = true;
        break;
      }
      lambda = __dmul_rn(lambda, 0.5);
    }
    if (!accepted) break;
  }
  *ox = x;
  *oy = y;
}

__device__ __forceinline__ void ref_ray(const Job& J, double u, double v, double ray[3]) {
  const double xn = __ddiv_rn(__dsub_rn(u, J.drcx), J.drfx);
  const double yn = __ddiv_rn(__dsub_rn(v, J.drcy), J.drfy);
  if (J.ref_distorted) {
    remove_distortion_d(J.rk1, J.rk2, J.rk3, J.rp1, J.rp2, xn, yn, &ray[0], &ray[1]);
  } else {
    ray[0] = xn;
    ray[1] = yn;
  }
  ray[2] = 1.0;
}

}  // namespace rmvs
