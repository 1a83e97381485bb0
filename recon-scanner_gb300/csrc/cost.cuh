// cost.cuh -- NCC window cost of one hypothesis against one source view.
//
// Two window models share the same NCC rules (patchmatch_stereo.cpp:214-274):
// a sample counts when both its reference and source positions are inside
// the image (SampleBilinear's rule, :78-86); fewer than K*K/2 valid samples
// or sqrt(var_r * var_s) < 1e-9 make the view invalid; NCC is clamped to
// [-1, 1].
//
//  * COMPAT -- the reference's own model (EvaluateCandidate, :344-418): a
//    fronto-parallel hypothesis; only the window centre is projected; the
//    source window is the reference window translated to the projected
//    centre; both images are read with index == coordinate, so the
//    reference window at pixel centres is the 2x2 box filter of the image.
//  * PLANE -- a plane hypothesis (inverse depth at the pixel centre + unit
//    normal): every sample (x+dx+0.5, y+dy+0.5) of the reference window is
//    mapped through the plane-induced homography into the source and read
//    with the pixel-centre convention (index == coordinate - 0.5).
//
// Per sample the PLANE path costs ~22 FP32 instructions, one MUFU.RCP, one
// texture gather (the 2x2 bilinear footprint) and one reference read;
// the window centre is computed once per (hypothesis, view) in float-float.
// Moments are accumulated on data centred per window (reference window mean,
// source centre sample) with per-row partial sums, which keeps FP32 NCC
// within ~1e-6 of an FP64 evaluation.
#pragma once

#include "common.cuh"

namespace rmvs {

struct ViewResult {
  float ncc;
  int valid;  // 1 valid; 0 invalid after sampling; -1 invalid before sampling (plane mode)
};

// Window moments of the reference image for one pixel (full window).
struct RefWindow {
  float mean;   // mean of (I - 128) over the window (the centring offset)
  float sxx;    // sum of squared centred values
  bool full;    // the whole K x K window lies inside the reference image
};

// Centre of the source window in float-float.  Xn = P + rho * b is the
// source-camera point scaled by rho (P = A * ray, computed once per pixel in
// FP64).  Returns false when the point is not in front of the camera
// (p_src.z <= 1e-6, patchmatch_stereo.cpp:391).
__device__ __forceinline__ bool source_centre(const SrcView& S, const ff P[3], ff rho, float rho_f, ff* u0,
                                              ff* v0, float* xz, float* mx, float* my) {
  const ff Xx = ff_add(P[0], ff_mul(S.bff[0], rho));
  const ff Xy = ff_add(P[1], ff_mul(S.bff[1], rho));
  const ff Xz = ff_add(P[2], ff_mul(S.bff[2], rho));
  // p_src.z = Xz / rho
  if (!(Xz.hi + Xz.lo > 1e-6f * rho_f)) return false;
  ff x = ff_div(Xx, Xz);
  ff y = ff_div(Xy, Xz);
  *xz = Xz.hi;
  *mx = x.hi;
  *my = y.hi;
  if (S.distorted) {
    // ApplyDistortion (camera.cpp:33-45) in float-float
    const ff x2 = ff_mul(x, x), y2 = ff_mul(y, y);
    const ff r2 = ff_add(x2, y2);
    const ff r4 = ff_mul(r2, r2);
    const ff r6 = ff_mul(r4, r2);
    ff radial = ff_add(ff_make(1.0f), ff_mul_f(r2, S.k1));
    radial = ff_add(radial, ff_mul_f(r4, S.k2));
    radial = ff_add(radial, ff_mul_f(r6, S.k3));
    const ff xy = ff_mul(x, y);
    const ff pxy = ff_add(ff_mul_f(xy, S.p1), ff_mul_f(ff_add(r2, ff_mul_f(x2, 2.0f)), S.p2));
    const ff pxy2 = ff_add(ff_mul_f(ff_add(r2, ff_mul_f(y2, 2.0f)), S.p1), ff_mul_f(xy, S.p2));
    x = ff_add(ff_mul(x, radial), pxy);
    y = ff_add(ff_mul(y, radial), pxy2);
  }
  *u0 = ff_add(ff_mul(S.ffx, x), S.fcx);
  *v0 = ff_add(ff_mul(S.ffy, y), S.fcy);
  return true;
}

// How plane-mode kernels read source texels (a template parameter, the
// constants kSrcExact / kSrcTex / kSrcBf16):
//   kSrcExact -- FP32 or FP16 texture, 2x2 gather, exact FP32 bilinear;
//   kSrcTex   -- the texture unit's bilinear filter (8-bit fixed-point weights);
//   kSrcBf16  -- BF16 values in a 16-bit unsigned texture (the texture unit has
//                no BF16 format), 2x2 gather of the raw bits widened exactly to
//                FP32, exact FP32 bilinear.

// The 2x2 footprint at gather coordinate (x, y); order (x0,y1) (x1,y1) (x1,y0) (x0,y0).
template <int kMode>
__device__ __forceinline__ float4 gather4(cudaTextureObject_t tex, float x, float y) {
  if constexpr (kMode == kSrcBf16) {
    const ushort4 g = tex2Dgather<ushort4>(tex, x, y, 0);
    return make_float4(__uint_as_float((unsigned)g.x << 16), __uint_as_float((unsigned)g.y << 16),
                       __uint_as_float((unsigned)g.z << 16), __uint_as_float((unsigned)g.w << 16));
  } else {
    return tex2Dgather<float4>(tex, x, y, 0);
  }
}

// Bilinear read of the 2x2 footprint whose top-left texel is (x0, y0),
// given as float texel indices.
template <int kMode = kSrcExact>
__device__ __forceinline__ float bilinear(cudaTextureObject_t tex, float x0, float y0, float fx, float fy) {
  const float4 g = gather4<kMode>(tex, x0 + 1.0f, y0 + 1.0f);
  const float top = fmaf(fx, g.z - g.w, g.w);
  const float bot = fmaf(fx, g.y - g.x, g.x);
  return fmaf(fy, bot - top, top);
}

// Kahan-compensated accumulation: sum += v with the running compensation c.
__device__ __forceinline__ void kahan_add(float& sum, float& c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(sum, y);
  c = __fsub_rn(__fsub_rn(t, sum), y);
  sum = t;
}

__device__ __forceinline__ ViewResult ncc_from_moments(float n, float sr, float srr, float ss, float sss, float srs,
                                                       int min_valid) {
  ViewResult r{0.0f, 0};
  if (n < (float)min_valid) return r;
  const float inv_n = 1.0f / n;
  const float mr = sr * inv_n, ms = ss * inv_n;
  const float var_r = srr * inv_n - mr * mr;
  const float var_s = sss * inv_n - ms * ms;
  const float denom = sqrtf(var_r * var_s);
  if (!(denom >= 1e-9f)) return r;
  float ncc = (srs * inv_n - mr * ms) / denom;
  ncc = fminf(1.0f, fmaxf(-1.0f, ncc));
  r.ncc = ncc;
  r.valid = 1;
  return r;
}

// ---------------------------------------------------------------------------
// COMPAT: translated window (reference semantics)
// ---------------------------------------------------------------------------
__device__ __forceinline__ ViewResult eval_view_compat(const Job& J, const SrcView& S, int x, int y, const ff P[3],
                                                       ff rho, float rho_f, const RefWindow& rw) {
  ViewResult bad{0.0f, 0};
  ff u0, v0;
  float xz, mx, my;
  if (!source_centre(S, P, rho, rho_f, &u0, &v0, &xz, &mx, &my)) return bad;
  int iu, iv;
  float fu, fv;
  ff_floor_frac(u0, &iu, &fu);
  ff_floor_frac(v0, &iv, &fv);
  const int h = J.patch_half;
  // valid rectangle: reference index x+0.5+dx in [0, W-1]; source index
  // u0+dx in [0, Ws-1] (dx, dy integers)
  const int dx_lo = max(-h, max(-x, -iu));
  const int dx_hi = min(h, min(J.w - 2 - x, (fu == 0.0f ? S.w - 1 : S.w - 2) - iu));
  const int dy_lo = max(-h, max(-y, -iv));
  const int dy_hi = min(h, min(J.h - 2 - y, (fv == 0.0f ? S.h - 1 : S.h - 2) - iv));
  const int nxv = dx_hi - dx_lo + 1, nyv = dy_hi - dy_lo + 1;
  const int K = 2 * h + 1;
  const int min_valid = J.min_valid;
  if (nxv <= 0 || nyv <= 0 || nxv * nyv < min_valid) return bad;
  // centre the source by its value at the window centre (or the nearest
  // valid sample)
  const int cdx = min(max(0, dx_lo), dx_hi), cdy = min(max(0, dy_lo), dy_hi);
  const float sc = bilinear(S.tex, (float)(iu + cdx), (float)(iv + cdy), fu, fv);
  const float rmean = rw.mean;
  float sr = 0.f, srr = 0.f, ss = 0.f, sss = 0.f, srs = 0.f;
  const bool full = rw.full && nxv == K && nyv == K;
  for (int dy = dy_lo; dy <= dy_hi; ++dy) {
    const float* rrow = J.ref_box + (size_t)(y + dy) * J.w + x;
    const float gy = (float)(iv + dy);
    float r_s = 0.f, r_ss = 0.f, r_rs = 0.f, r_r = 0.f, r_rr = 0.f;
    for (int dx = dx_lo; dx <= dx_hi; ++dx) {
      const float rv = __ldg(rrow + dx) - rmean;
      const float sv = bilinear(S.tex, (float)(iu + dx), gy, fu, fv) - sc;
      r_s += sv;
      r_ss = fmaf(sv, sv, r_ss);
      r_rs = fmaf(rv, sv, r_rs);
      if (!full) {
        r_r += rv;
        r_rr = fmaf(rv, rv, r_rr);
      }
    }
    ss += r_s;
    sss += r_ss;
    srs += r_rs;
    sr += r_r;
    srr += r_rr;
  }
  if (full) {
    sr = 0.0f;
    srr = rw.sxx;
  }
  return ncc_from_moments((float)(nxv * nyv), sr, srr, ss, sss, srs, min_valid);
}

// ---------------------------------------------------------------------------
// PLANE: homography window
// ---------------------------------------------------------------------------
struct PlaneHyp {
  float rho;          // inverse depth at the pixel centre
  float nx, ny, nz;   // unit normal, reference camera frame
  float kappa;        // n . ray(pixel centre)  (< 0 for a plane facing the camera)
  float s0, s1;       // rho * nx / (fx kappa), rho * ny / (fy kappa)
  float ex, ey;       // nx / fx, ny / fy   (n . ray changes by ex per dx)
};

__device__ __forceinline__ bool make_plane_hyp(const Job& J, float rx, float ry, float rho, float nx, float ny,
                                               float nz, PlaneHyp* hp) {
  const float kappa = nx * rx + ny * ry + nz;  // ray z = 1
  // grazing or back-facing planes are not hypotheses
  const float rn = sqrtf(rx * rx + ry * ry + 1.0f);
  if (!(kappa < -0.05f * rn)) return false;
  hp->rho = rho;
  hp->nx = nx;
  hp->ny = ny;
  hp->nz = nz;
  hp->kappa = kappa;
  hp->ex = nx / J.rfx;
  hp->ey = ny / J.rfy;
  hp->s0 = rho * hp->ex / kappa;
  hp->s1 = rho * hp->ey / kappa;
  return true;
}

template <bool kFull, int kMode>
__device__ __forceinline__ void plane_window(const Job& J, const SrcView& S, int x, int y, int iu, int iv, float fu,
                                             float fv, float A0, float A1, float B0, float B1, float c0, float c1,
                                             const PlaneHyp& hp, float rmean, float sc, float* acc, float* cnt) {
  const int h = J.patch_half;
  float sr = 0.f, srr = 0.f, ss = 0.f, sss = 0.f, srs = 0.f, n = 0.f;
  float cr = 0.f, crr = 0.f, cs = 0.f, css = 0.f, crs = 0.f;  // Kahan compensations across rows
  const float bu = (float)iu, bv = (float)iv;
  const float umax = (float)(S.w - 1 - iu), vmax = (float)(S.h - 1 - iv);
  const float umin = (float)(-iu), vmin = (float)(-iv);
  for (int dy = -h; dy <= h; ++dy) {
    const int ry = y + dy;
    if (!kFull && (ry < 0 || ry > J.h - 1 - J.half_pixel)) continue;
    const float fdy = (float)dy;
    float den = fmaf(fdy, c1, 1.0f - (float)h * c0);
    float nu = fmaf(fdy, A1, -(float)h * A0);
    float nv = fmaf(fdy, B1, -(float)h * B0);
    float nr = hp.kappa + fdy * hp.ey - (float)h * hp.ex;
    const float* rrow = J.pref + (size_t)ry * J.w + x;
    float r_s = 0.f, r_ss = 0.f, r_rs = 0.f, r_r = 0.f, r_rr = 0.f, r_n = 0.f;
#pragma unroll 4
    for (int dx = -h; dx <= h; ++dx) {
      const float rinv = __frcp_rn(den);
      const float tu = fmaf(nu, rinv, fu);
      const float tv = fmaf(nv, rinv, fv);
      bool ok = true;
      if (!kFull) {
        const int rx = x + dx;
        ok = rx >= 0 && rx <= J.w - 1 - J.half_pixel && den > 0.0f && nr < 0.0f && tu >= umin && tu <= umax && tv >= vmin &&
             tv <= vmax;
      }
      if (ok) {
        const float flu = floorf(tu), flv = floorf(tv);
        const float sv = (kMode == kSrcTex ? tex2D<float>(S.tex_lin, bu + tu + 0.5f, bv + tv + 0.5f)
                                           : bilinear<kMode>(S.tex, bu + flu, bv + flv, tu - flu, tv - flv)) - sc;
        const float rv = __ldg(rrow + dx) - rmean;
        r_s += sv;
        r_ss = fmaf(sv, sv, r_ss);
        r_rs = fmaf(rv, sv, r_rs);
        if (!kFull) {
          r_r += rv;
          r_rr = fmaf(rv, rv, r_rr);
          r_n += 1.0f;
        }
      }
      den += c0;
      nu += A0;
      nv += B0;
      nr += hp.ex;
    }
    kahan_add(ss, cs, r_s);
    kahan_add(sss, css, r_ss);
    kahan_add(srs, crs, r_rs);
    kahan_add(sr, cr, r_r);
    kahan_add(srr, crr, r_rr);
    n += r_n;
  }
  acc[0] = sr;
  acc[1] = srr;
  acc[2] = ss;
  acc[3] = sss;
  acc[4] = srs;
  *cnt = n;
}

// Reference-window accessors for the unrolled window: value of sample
// k = dx + H of a row, split into even k (even(m), k = 2m) and odd k
// (odd(m), k = 2m + 1) so that, with H known at compile time, every offset
// is a constant.
struct GlobalRow {
  const float* p;  // row start at x - H
  __device__ __forceinline__ float even(int m) const { return __ldg(p + 2 * m); }
  __device__ __forceinline__ float odd(int m) const { return __ldg(p + 2 * m + 1); }
};

struct GlobalRef {
  const float* ref;
  int w, x, y;
  template <int H>
  __device__ __forceinline__ GlobalRow row(int dy) const {
    return GlobalRow{ref + (size_t)(y + dy) * w + (x - H)};
  }
};

// Shared-memory tile of the reference image stored as even / odd column
// planes, so that the lanes of a warp (same-colour pixels two columns apart,
// 8 per row in 4 rows) read consecutive words of 4 rows whose pitch puts them
// in distinct banks: conflict-free.

struct TileRow {
  const float* a;
  const float* b;
  __device__ __forceinline__ float even(int m) const { return a[m]; }
  __device__ __forceinline__ float odd(int m) const { return b[m]; }
};

struct TileRef {
  const float* same;   // the column plane of this thread's own parity, [rows][kTileCols]
  const float* other;  // the other plane
  int pair, parity, ty;  // the pixel's column pair and row in the tile
  template <int H>
  __device__ __forceinline__ TileRow row(int dy) const {
    const int r = (ty + H + dy) * kTileCols + pair + 8;
    if (H & 1) return TileRow{other + r + parity - (H + 1) / 2, same + r - (H - 1) / 2};
    return TileRow{same + r - H / 2, other + r + parity - H / 2};
  }
};

// How the exact fast path reads a sample's 2x2 footprint.  The argument is
// the footprint's top-left texel relative to the window centre's texel
// (iu, iv), as the floats mu, mv = n + kM (kM = 1.5 * 2^23, so that the
// integer n sits in the low mantissa bits).  Both return the footprint in
// gather order: (x0,y1) (x1,y1) (x1,y0) (x0,y0).
constexpr float kMagic = 12582912.0f;
constexpr unsigned kMagicBits = 0x4B400000u;  // __float_as_uint(kMagic)

template <int kMode>
struct TexGather {  // one 2x2 gather from the source texture
  cudaTextureObject_t tex;
  float gxo, gyo;  // (iu + 1) - kM, (iv + 1) - kM: the gather coordinates are exact integers
  __device__ __forceinline__ float4 operator()(float mu, float mv) const {
    return gather4<kMode>(tex, __fadd_rn(mu, gxo), __fadd_rn(mv, gyo));
  }
};

template <int kMode>
__device__ __forceinline__ TexGather<kMode> tex_gather(cudaTextureObject_t tex, int iu, int iv) {
  return TexGather<kMode>{tex, ((float)iu + 1.0f) - kMagic, ((float)iv + 1.0f) - kMagic};
}

// Two 8-byte loads of texel pairs from a warp's staged box (kStageH rows of
// kStageW pairs {T(x), T(x + 1)}, top-left texel (ax, ay)): the same four
// texels as the gather.  The element index is clamped into the box, so no
// read can leave it whatever the coordinates.
struct BoxFetch {
  const float2* box;
  unsigned base;  // element of the centre texel (iu, iv), less kMagicBits * (kStageW + 1)
  __device__ __forceinline__ float4 operator()(float mu, float mv) const {
    unsigned i = __float_as_uint(mv) * (unsigned)kStageW + __float_as_uint(mu) + base;
    i = min(i, (unsigned)(kStageW * (kStageH - 1) - 1));
    const float2 t = box[i], b = box[i + kStageW];
    return make_float4(b.x, b.y, t.y, t.x);
  }
};

__device__ __forceinline__ BoxFetch box_fetch(const float2* box, int ax, int ay, int iu, int iv) {
  return BoxFetch{box, (unsigned)((iv - ay) * kStageW + (iu - ax)) - kMagicBits * (unsigned)(kStageW + 1)};
}

// The bilinear value at fraction (fx, fy) of the footprint whose top-left
// texel is the window centre's own: bilinear()'s arithmetic on a fetch.
template <class Fetch>
__device__ __forceinline__ float centre_sample(const Fetch& f, float fx, float fy) {
  const float4 g = f(kMagic, kMagic);
  const float top = fmaf(fx, g.z - g.w, g.w);
  const float bot = fmaf(fx, g.y - g.x, g.x);
  return fmaf(fy, bot - top, top);
}

// One window row of the fast path, fully unrolled.  Floors by magic-number
// rounding (FMA pipe): m = t' + 1.5*2^23 rounds t' = t - 0.5 to the nearest
// integer, i.e. floor(t); at exact ties the footprint shifts by one texel
// with weight 1, which reads the same value (bilinear is continuous).
template <int H, int kMode, class Row, class Fetch>
__device__ __forceinline__ void plane_row(const Fetch& fetch, cudaTextureObject_t tex_lin, const Row& row,
                                          float& den, float& nu, float& nv, float c0, float A0, float B0, float fum,
                                          float fvm, float cuo, float cvo, float rmean, float sc, float& r_s,
                                          float& r_ss, float& r_rs) {
  constexpr float kM = 12582912.0f;
#pragma unroll
  for (int k = 0; k <= 2 * H; ++k) {
    const float rinv = rcp_approx(den);
    float sv;
    if constexpr (kMode == kSrcTex) {
      // texture coordinate of index coordinate t: t + 0.5
      sv = tex2D<float>(tex_lin, fmaf(nu, rinv, cuo), fmaf(nv, rinv, cvo)) - sc;
    } else {
      const float tmu = fmaf(nu, rinv, fum);
      const float tmv = fmaf(nv, rinv, fvm);
      const float mu = __fadd_rn(tmu, kM), mv = __fadd_rn(tmv, kM);
      const float flu = __fsub_rn(mu, kM), flv = __fsub_rn(mv, kM);
      const float wu = __fadd_rn(__fsub_rn(tmu, flu), 0.5f);
      const float wv = __fadd_rn(__fsub_rn(tmv, flv), 0.5f);
      const float4 g = fetch(mu, mv);
      const float top = fmaf(wu, g.z - g.w, g.w);
      const float bot = fmaf(wu, g.y - g.x, g.x);
      sv = fmaf(wv, bot - top, top) - sc;
    }
    const float rv = ((k & 1) ? row.odd(k >> 1) : row.even(k >> 1)) - rmean;
    r_s += sv;
    r_ss = fmaf(sv, sv, r_ss);
    r_rs = fmaf(rv, sv, r_rs);
    den += c0;
    nu += A0;
    nv += B0;
  }
}

// The moments of a window that straddles a source border (reference part
// inside the image, plane facing the camera): each sample carries a validity
// mask -- its source position inside [0, w-1] x [0, h-1] -- and the reference
// moments are accumulated too.  Plane-side and denominator signs need no
// per-sample test: they are affine in (dx, dy) and the corner test found them
// right at all four corners.  Rows are combined with Kahan-compensated sums.
template <int H, int kMode, class Ref>
__device__ __forceinline__ void plane_window_masked(const SrcView& S, const Ref& ref, int iu, int iv, float fu,
                                                    float fv, float A0, float A1, float B0, float B1, float c0,
                                                    float c1, float rmean, float sc, float* acc, float* cnt) {
  constexpr float kM = 12582912.0f;
  // validity bounds of the index coordinate relative to texel (iu, iv)
  const float lu = (float)(-iu), hu = (float)(S.w - 1 - iu), lv = (float)(-iv), hv = (float)(S.h - 1 - iv);
  const float gxo = ((float)iu + 1.0f) - kM, gyo = ((float)iv + 1.0f) - kM;
  const float cuo = ((float)iu + 0.5f), cvo = ((float)iv + 0.5f);
  float ss = 0.f, sss = 0.f, srs = 0.f, sr = 0.f, srr = 0.f, n = 0.f;
  float cs = 0.f, css = 0.f, crs = 0.f, cr = 0.f, crr = 0.f;
#pragma unroll 1
  for (int dy = -H; dy <= H; ++dy) {
    const auto row = ref.template row<H>(dy);
    const float fdy = (float)dy;
    float den = fmaf(fdy, c1, fmaf(-(float)H, c0, 1.0f));
    float nu = fmaf(fdy, A1, -(float)H * A0);
    float nv = fmaf(fdy, B1, -(float)H * B0);
    float r_s = 0.f, r_ss = 0.f, r_rs = 0.f, r_r = 0.f, r_rr = 0.f, r_n = 0.f;
#pragma unroll 1
    for (int k = 0; k <= 2 * H; ++k) {
      const float rinv = rcp_approx(den);
      const float tu = fmaf(nu, rinv, fu), tv = fmaf(nv, rinv, fv);  // relative index coordinates
      den += c0;
      nu += A0;
      nv += B0;
      if (!(tu >= lu && tu <= hu && tv >= lv && tv <= hv)) continue;
      float sv;
      if constexpr (kMode == kSrcTex) {
        sv = tex2D<float>(S.tex_lin, tu + cuo, tv + cvo) - sc;
      } else {
        const float mu = __fadd_rn(tu - 0.5f, kM), mv = __fadd_rn(tv - 0.5f, kM);
        const float flu = __fsub_rn(mu, kM), flv = __fsub_rn(mv, kM);
        sv = bilinear<kMode>(S.tex, __fadd_rn(mu, gxo) - 1.0f, __fadd_rn(mv, gyo) - 1.0f, tu - flu, tv - flv) - sc;
      }
      const float rv = ((k & 1) ? row.odd(k >> 1) : row.even(k >> 1)) - rmean;
      r_s += sv;
      r_ss = fmaf(sv, sv, r_ss);
      r_rs = fmaf(rv, sv, r_rs);
      r_r += rv;
      r_rr = fmaf(rv, rv, r_rr);
      r_n += 1.0f;
    }
    kahan_add(ss, cs, r_s);
    kahan_add(sss, css, r_ss);
    kahan_add(srs, crs, r_rs);
    kahan_add(sr, cr, r_r);
    kahan_add(srr, crr, r_rr);
    n += r_n;
  }
  acc[0] = sr;
  acc[1] = srr;
  acc[2] = ss;
  acc[3] = sss;
  acc[4] = srs;
  *cnt = n;
}

// The moments of a full window: each row's partial sums in plain FP32 (11
// terms), the rows combined with Kahan-compensated sums.
template <int H, int kMode, class Ref, class Fetch>
__device__ __forceinline__ void plane_window_fast(const Fetch& fetch, cudaTextureObject_t tex_lin, const Ref& ref,
                                                  int iu, int iv, float fu, float fv, float A0, float A1, float B0,
                                                  float B1, float c0, float c1, float rmean, float sc, float* acc) {
  const float fum = fu - 0.5f, fvm = fv - 0.5f;
  const float cuo = ((float)iu + 0.5f) + fu, cvo = ((float)iv + 0.5f) + fv;
  float ss = 0.f, sss = 0.f, srs = 0.f;
  float cs = 0.f, css = 0.f, crs = 0.f;
#pragma unroll 1
  for (int dy = -H; dy <= H; ++dy) {
    const float fdy = (float)dy;
    float den = fmaf(fdy, c1, fmaf(-(float)H, c0, 1.0f));
    float nu = fmaf(fdy, A1, -(float)H * A0);
    float nv = fmaf(fdy, B1, -(float)H * B0);
    float r_s = 0.f, r_ss = 0.f, r_rs = 0.f;
    plane_row<H, kMode>(fetch, tex_lin, ref.template row<H>(dy), den, nu, nv, c0, A0, B0, fum, fvm, cuo, cvo, rmean,
                        sc, r_s, r_ss, r_rs);
    kahan_add(ss, cs, r_s);
    kahan_add(sss, css, r_ss);
    kahan_add(srs, crs, r_rs);
  }
  acc[2] = ss;
  acc[3] = sss;
  acc[4] = srs;
}

// The window's moments as the adjoint wants them: n, the means of the
// reference and source values, and the centred sums of squares and products
// -- from sums shifted by (rmean, sc): mean = shift + S / n, centred =
// S2 - S S' / n.
__device__ __forceinline__ void window_moments(float* mom, float n, float rmean, float sc, float sr, float srr,
                                               float ss, float sss, float srs) {
  const float inv_n = 1.0f / n;
  mom[0] = n;
  mom[1] = rmean + sr * inv_n;
  mom[2] = sc + ss * inv_n;
  mom[3] = srr - sr * sr * inv_n;
  mom[4] = sss - ss * ss * inv_n;
  mom[5] = srs - sr * ss * inv_n;
}

// Where a plane hypothesis' window falls in one source: the per-sample
// offsets from the window centre, du = (dx A0 + dy A1) / (1 + dx c0 + dy c1)
// (dv likewise with B), the centre's texel (iu, iv) and fraction (fu, fv) in
// the pixel-centre convention (index coordinate = coordinate - 0.5), and the
// four corners' index coordinates relative to (iu, iv).
struct WindowPlace {
  float A0, A1, B0, B1, c0, c1;
  int iu, iv;
  float fu, fv;
  float umin, umax, vmin, vmax;
  bool full;     // the whole window inside the source, in front of it, on the camera side of the plane
  bool front;    // the four corners in front of the source and on the camera side of the plane
  bool outside;  // in front, and every corner beyond one image edge: no sample is valid
};

// False when the window centre is not in front of the source (nothing is
// sampled).  The four corners decide the window: all inside (and in front of
// the source, on the camera side of the plane) -> every sample is valid, by
// convexity of the projective image of the window; all beyond one image edge
// -> no sample is valid and the view is invalid without sampling.
template <int H>
__device__ __forceinline__ bool place_window(const Job& J, const SrcView& S, const ff P[3], const PlaneHyp& hp,
                                              const RefWindow& rw, WindowPlace* g) {
  ff u0, v0;
  float xz, mx, my;
  if (!source_centre(S, P, ff_make(hp.rho), hp.rho, &u0, &v0, &xz, &mx, &my)) return false;
  const float G0x = fmaf(hp.s0, S.b[0], S.Ac0[0]);
  const float G0y = fmaf(hp.s0, S.b[1], S.Ac0[1]);
  const float G0z = fmaf(hp.s0, S.b[2], S.Ac0[2]);
  const float G1x = fmaf(hp.s1, S.b[0], S.Ac1[0]);
  const float G1y = fmaf(hp.s1, S.b[1], S.Ac1[1]);
  const float G1z = fmaf(hp.s1, S.b[2], S.Ac1[2]);
  const float iz = rcp_approx(xz);
  g->A0 = S.fx * (G0x - mx * G0z) * iz;
  g->A1 = S.fx * (G1x - mx * G1z) * iz;
  g->B0 = S.fy * (G0y - my * G0z) * iz;
  g->B1 = S.fy * (G1y - my * G1z) * iz;
  g->c0 = G0z * iz;
  g->c1 = G1z * iz;
  const float shift = J.half_pixel ? 0.0f : -0.5f;
  ff_floor_frac(ff_add(u0, ff_make(shift)), &g->iu, &g->fu);
  ff_floor_frac(ff_add(v0, ff_make(shift)), &g->iv, &g->fv);
  const int h = H > 0 ? H : J.patch_half;
  const float fh = (float)h;
  bool front = true;
  float umin_c = 3.4e38f, umax_c = -3.4e38f, vmin_c = 3.4e38f, vmax_c = -3.4e38f;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float dx = (c & 1) ? fh : -fh, dy = (c & 2) ? fh : -fh;
    const float den = fmaf(dx, g->c0, fmaf(dy, g->c1, 1.0f));
    const float rd = rcp_approx(den);
    const float tu = g->fu + fmaf(dx, g->A0, dy * g->A1) * rd;
    const float tv = g->fv + fmaf(dx, g->B0, dy * g->B1) * rd;
    const float nr = hp.kappa + dx * hp.ex + dy * hp.ey;
    front = front && den > 0.0f && nr < 0.0f;
    umin_c = fminf(umin_c, tu);
    umax_c = fmaxf(umax_c, tu);
    vmin_c = fminf(vmin_c, tv);
    vmax_c = fmaxf(vmax_c, tv);
  }
  const float ulo = (float)(-g->iu), uhi = (float)(S.w - 1 - g->iu), vlo = (float)(-g->iv),
              vhi = (float)(S.h - 1 - g->iv);
  g->front = front;
  g->full = rw.full && front && umin_c >= ulo + 0.001f && umax_c <= uhi - 0.001f && vmin_c >= vlo + 0.001f &&
            vmax_c <= vhi - 0.001f;
  g->outside = front && (umax_c < ulo - 0.001f || umin_c > uhi + 0.001f || vmax_c < vlo - 0.001f ||
                         vmin_c > vhi + 0.001f);
  g->umin = umin_c;
  g->umax = umax_c;
  g->vmin = vmin_c;
  g->vmax = vmax_c;
  return true;
}

// The NCC of a window placed by place_window, its samples read from the
// source texture.
template <int H, int kMode, class Ref>
__device__ __forceinline__ ViewResult eval_view_placed(const Job& J, const SrcView& S, int x, int y, const WindowPlace& g,
                                                    const PlaneHyp& hp, const RefWindow& rw, const Ref& ref,
                                                    float* mom = nullptr) {
  ViewResult bad{0.0f, -1};  // nothing sampled
  const int iu = g.iu, iv = g.iv;
  const float fu = g.fu, fv = g.fv;
  // source centring value: the sample at the window centre (clamped read)
  const float sc = kMode == kSrcTex ? tex2D<float>(S.tex_lin, (float)iu + 0.5f + fu, (float)iv + 0.5f + fv)
                                    : bilinear<kMode>(S.tex, (float)iu, (float)iv, fu, fv);
  float acc[5], n;
  const int h = H > 0 ? H : J.patch_half;
  const int K = 2 * h + 1;
  const int min_valid = J.min_valid;
  if (g.outside) return bad;
  if constexpr (H > 0) {
    if (g.full) {
      plane_window_fast<H, kMode>(tex_gather<kMode>(S.tex, iu, iv), S.tex_lin, ref, iu, iv, fu, fv, g.A0, g.A1, g.B0,
                                  g.B1, g.c0, g.c1, rw.mean, sc, acc);
      if (mom) window_moments(mom, (float)(K * K), rw.mean, sc, 0.0f, rw.sxx, acc[2], acc[3], acc[4]);
      return ncc_from_moments((float)(K * K), 0.0f, rw.sxx, acc[2], acc[3], acc[4], min_valid);
    }
    if (rw.full && g.front) {
      // straddles a source border: masked samples, reference from the tile
      plane_window_masked<H, kMode>(S, ref, iu, iv, fu, fv, g.A0, g.A1, g.B0, g.B1, g.c0, g.c1, rw.mean, sc, acc,
                                    &n);
      if (mom && n > 0.f) window_moments(mom, n, rw.mean, sc, acc[0], acc[1], acc[2], acc[3], acc[4]);
      return ncc_from_moments(n, acc[0], acc[1], acc[2], acc[3], acc[4], min_valid);
    }
  } else if (g.full) {
    plane_window<true, kMode>(J, S, x, y, iu, iv, fu, fv, g.A0, g.A1, g.B0, g.B1, g.c0, g.c1, hp, rw.mean, sc, acc,
                              &n);
    if (mom) window_moments(mom, (float)(K * K), rw.mean, sc, 0.0f, rw.sxx, acc[2], acc[3], acc[4]);
    return ncc_from_moments((float)(K * K), 0.0f, rw.sxx, acc[2], acc[3], acc[4], min_valid);
  }
  plane_window<false, kMode>(J, S, x, y, iu, iv, fu, fv, g.A0, g.A1, g.B0, g.B1, g.c0, g.c1, hp, rw.mean, sc, acc,
                             &n);
  if (mom && n > 0.f) window_moments(mom, n, rw.mean, sc, acc[0], acc[1], acc[2], acc[3], acc[4]);
  return ncc_from_moments(n, acc[0], acc[1], acc[2], acc[3], acc[4], min_valid);
}

// The NCC of one hypothesis against one source view.  H > 0: windows of
// 2H+1 known at compile time, reference samples through `ref` on the fast
// path; H == 0: any window size (runtime loop).  The window's moments as the
// adjoint wants them (`mom`, optional): n, the means of the reference and
// source values, and the centred sums of squares and products.
template <int H, int kMode, class Ref>
__device__ __forceinline__ ViewResult eval_view_plane(const Job& J, const SrcView& S, int x, int y, const ff P[3],
                                                      const PlaneHyp& hp, const RefWindow& rw, const Ref& ref,
                                                      float* mom = nullptr) {
  WindowPlace g;
  if (!place_window<H>(J, S, P, hp, rw, &g)) return ViewResult{0.0f, -1};
  return eval_view_placed<H, kMode>(J, S, x, y, g, hp, rw, ref, mom);
}

// The NCC of a full window (place_window's `full`) whose samples are read
// from a warp's staged box: the fast path's arithmetic, footprints from the
// box instead of the texture -- the same value as eval_view_placed, bit for bit.
template <int H, class Ref>
__device__ __forceinline__ ViewResult eval_view_box(const Job& J, const WindowPlace& g, const RefWindow& rw, const Ref& ref,
                                                    const float2* box, int ax, int ay) {
  const BoxFetch f = box_fetch(box, ax, ay, g.iu, g.iv);
  const float sc = centre_sample(f, g.fu, g.fv);
  float acc[5];
  constexpr int K = 2 * H + 1;
  plane_window_fast<H, kSrcExact>(f, 0, ref, g.iu, g.iv, g.fu, g.fv, g.A0, g.A1, g.B0, g.B1, g.c0, g.c1, rw.mean, sc,
                                  acc);
  return ncc_from_moments((float)(K * K), 0.0f, rw.sxx, acc[2], acc[3], acc[4], J.min_valid);
}

// Reference-window statistics for a pixel: mean and centred sum of squares of
// (I - 128) over the full K x K window (compat: of the box-filtered image).
__device__ __forceinline__ RefWindow ref_window(const Job& J, int x, int y, bool compat) {
  RefWindow rw;
  const int h = J.patch_half;
  const int wlim = compat ? J.w - 2 : J.w - 1;
  const int hlim = compat ? J.h - 2 : J.h - 1;
  const float* img = compat ? J.ref_box : J.ref;
  int x0 = max(0, x - h), x1 = min(wlim, x + h), y0 = max(0, y - h), y1 = min(hlim, y + h);
  rw.full = (x0 == x - h && x1 == x + h && y0 == y - h && y1 == y + h);
  float s = 0.f;
  int n = 0;
  for (int yy = y0; yy <= y1; ++yy)
    for (int xx = x0; xx <= x1; ++xx) {
      s += __ldg(img + (size_t)yy * J.w + xx);
      ++n;
    }
  rw.mean = n > 0 ? s / (float)n : 0.0f;
  float q = 0.f;
  for (int yy = y0; yy <= y1; ++yy) {
    float qr = 0.f;
    for (int xx = x0; xx <= x1; ++xx) {
      const float d = __ldg(img + (size_t)yy * J.w + xx) - rw.mean;
      qr = fmaf(d, d, qr);
    }
    q += qr;
  }
  rw.sxx = q;
  return rw;
}

// P = A * ray for every source of the job, FP64 -> float-float.
__device__ __forceinline__ void source_rays(const Job& J, const SrcView& S, const double ray[3], ff P[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double v = S.A[i * 3 + 0] * ray[0] + S.A[i * 3 + 1] * ray[1] + S.A[i * 3 + 2] * ray[2];
    P[i] = ff_from_double(v);
  }
}

}  // namespace rmvs
