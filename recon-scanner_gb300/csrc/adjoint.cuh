// adjoint.cuh -- the hand-written adjoint of the aggregated plane cost.
//
// Parameters.  A pixel's hypothesis is (d, theta, phi): the depth d of the
// plane at the pixel-centre ray (z = d) and the unit normal
//   n = (sin t cos p, sin t sin p, cos t)
// in the reference camera frame.  A source's pose enters through the
// relative transform Y = A X + b (reference camera -> source camera),
// perturbed on the left in the source frame: Y' = exp([w]x) Y + tau, so the
// 6 pose parameters are (w, tau).
//
// Forward.  Window sample k at reference pixel (x+dx, y+dy) with ray q_k:
//   X_k = q_k * d kappa / m_k,  kappa = n . q_c,  m_k = n . q_k
//   Y_k = A X_k + b,  (u, v) = (fx Y.x / Y.z + cx, fy Y.y / Y.z + cy)
//   s_k = bilinear source read at (u - 0.5, v - 0.5) (pixel-centre convention)
// per view c = 1 - NCC(r, s) over the valid samples; the aggregated cost is
// the mean of the best_k view costs.
//
// Reverse.  With centred r~, s~ and S_rr, S_ss, NCC:
//   dc / ds_k = NCC s~_k / S_ss - r~_k / sqrt(S_rr S_ss)
// and ds_k/dp = grad I . dY/dp, so each view needs a second pass over its
// window (the window is recomputed, never stored) accumulating, per
// parameter vector d_k = ds_k/dp:  sum d, sum d d^T, sum s~ d and the
// residual sum sum e d with e_k = rho s~_k - r~_k, rho = NCC sqrt(S_rr / S_ss).
// Then
//   grad c = (NCC / S_ss) sum s~ d - sum r~ d / sqrt(S_rr S_ss)
//          = sum e d / sqrt(S_rr S_ss)
// -- the second form is what is computed: near a good match the two terms of
// the first nearly cancel (their FP32 rounding would swamp the gradient),
// while e_k is small per sample and its sum has no such cancellation.
// and the Gauss-Newton matrix of the equivalent residual form
// c = 1/2 sum_k (s^_k - r^_k)^2 (unit-normalised centred windows) is
//   H = [sum d d^T - n m m^T - (sum s~ d)(sum s~ d)^T / S_ss] / S_ss,  m = sum d / n.
// Sums are FP32 with Kahan compensation across window rows.
#pragma once

#include "cost.cuh"

namespace rmvs {

constexpr int kPoseH = 21;  // upper triangle of the 6 x 6 pose matrix

__device__ __forceinline__ void sph_normal(float t, float p, float n[3], float nt[3], float np[3]) {
  float st, ct, sp, cp;
  sincosf(t, &st, &ct);
  sincosf(p, &sp, &cp);
  n[0] = st * cp;
  n[1] = st * sp;
  n[2] = ct;
  nt[0] = ct * cp;
  nt[1] = ct * sp;
  nt[2] = -st;
  np[0] = -st * sp;
  np[1] = st * cp;
  np[2] = 0.0f;
}

// The hypothesis of one pixel in reference-camera terms.
struct AdjHyp {
  int x, y;
  float d, id;  // depth and 1 / depth
  float n[3], nt[3], np[3];
  float qc[3];  // pixel-centre ray
  float kappa;  // n . qc
  float irfx, irfy;  // 1 / reference focal lengths: ray offsets dx / fx, dy / fy
};

// Per-view moments of the first pass (values shifted by the window-centre
// samples, which leaves the NCC unchanged and keeps FP32 sums small).
struct ViewMom {
  float n, mr, ms, srr, sss, srs, ncc;
  bool valid;
};

// One view's geometry at a hypothesis: the window centre projected in
// float-float
// (index coordinates split into an integer texel and an FP32 fraction) and
// the FP32 transform for the offsets.  Samples are placed as centre +
// offset, the offset computed in FP32 from differences of small quantities,
// so a sample position is accurate to ~1e-6 px at any image coordinate.
struct ViewGeo {
  float A[9];
  float Yc[3];    // window-centre point, source camera
  float izc;      // 1 / Yc.z
  int iu, iv;     // texel of the centre (index coordinate = coordinate - 0.5)
  float fu, fv;   // its fraction
  bool ok;        // centre in front of the source (the search's rule)
};

__device__ __forceinline__ ViewGeo view_geo(const Job& J, const SrcView& S, const AdjHyp& h) {
  ViewGeo g;
#pragma unroll
  for (int i = 0; i < 9; ++i) g.A[i] = S.Aff[i].hi;
  // the window centre in float-float: X = q_c d, Y = A X + b, (u, v)
  const ff d = ff_make(h.d);
  const ff qx = ff_div(ff_add(ff_make((float)h.x + 0.5f), ff{-J.ffrcx.hi, -J.ffrcx.lo}), J.ffrx);
  const ff qy = ff_div(ff_add(ff_make((float)h.y + 0.5f), ff{-J.ffrcy.hi, -J.ffrcy.lo}), J.ffry);
  const ff X[3] = {ff_mul(qx, d), ff_mul(qy, d), d};
  ff Y[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    Y[i] = ff_add(ff_add(ff_add(ff_mul(S.Aff[3 * i], X[0]), ff_mul(S.Aff[3 * i + 1], X[1])),
                         ff_mul(S.Aff[3 * i + 2], X[2])),
                  S.bff[i]);
  g.ok = Y[2].hi > 1e-6f;
  int iu = 0, iv = 0;
  float fu = 0.f, fv = 0.f;
  if (g.ok) {
    const ff u = ff_add(ff_mul(S.ffx, ff_div(Y[0], Y[2])), ff_add(S.fcx, ff_make(-0.5f)));
    const ff v = ff_add(ff_mul(S.ffy, ff_div(Y[1], Y[2])), ff_add(S.fcy, ff_make(-0.5f)));
    g.ok = fabsf(u.hi) < 1e7f && fabsf(v.hi) < 1e7f;
    if (g.ok) {
      ff_floor_frac(u, &iu, &fu);
      ff_floor_frac(v, &iv, &fv);
    }
  }
  g.iu = iu;
  g.iv = iv;
  g.fu = fu;
  g.fv = fv;
#pragma unroll
  for (int i = 0; i < 3; ++i) g.Yc[i] = __fadd_rn(Y[i].hi, Y[i].lo);
  g.izc = 1.0f / g.Yc[2];
  return g;
}

// One window sample: returns false when invalid.  On success s = source
// value, r = reference value, X / Y = the plane point in the reference /
// source camera, G = dI/dY, m = n . q_k and q = the sample's ray (x, y).
template <int kMode, bool kGrad>
__device__ __forceinline__ bool adj_sample(const Job& J, const SrcView& S, const ViewGeo& geo, const AdjHyp& h,
                                           int dx, int dy, float* s, float* r, float X[3], float Y[3], float G[3],
                                           float* mk, float q[2]) {
  const int rx = h.x + dx, ry = h.y + dy;
  if (rx < 0 || ry < 0 || rx > J.w - 1 || ry > J.h - 1) return false;
  const float dq0 = (float)dx * h.irfx, dq1 = (float)dy * h.irfy;
  const float ndq = fmaf(h.n[0], dq0, h.n[1] * dq1);
  const float m = h.kappa + ndq;
  if (!(m < 0.0f)) return false;
  // X_k - X_c = d (kappa dq - (n . dq) q_c) / m_k   (exact small quantities)
  const float sc = h.d * rcp_approx(m);
  const float dX[3] = {sc * fmaf(h.kappa, dq0, -ndq * h.qc[0]), sc * fmaf(h.kappa, dq1, -ndq * h.qc[1]), -sc * ndq};
  float dY[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) dY[i] = fmaf(geo.A[i * 3], dX[0], fmaf(geo.A[i * 3 + 1], dX[1], geo.A[i * 3 + 2] * dX[2]));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Y[i] = geo.Yc[i] + dY[i];
    X[i] = fmaf(h.d, h.qc[i], dX[i]);
  }
  if (!(Y[2] > 1e-9f)) return false;
  const float iz = rcp_approx(Y[2]);
  const float izc = geo.izc;
  // offset from the centre in index coordinates
  const float du = S.fx * fmaf(dY[0], geo.Yc[2], -geo.Yc[0] * dY[2]) * (iz * izc);
  const float dv = S.fy * fmaf(dY[1], geo.Yc[2], -geo.Yc[1] * dY[2]) * (iz * izc);
  const float tu = geo.fu + du, tv = geo.fv + dv;
  const float fl_u = floorf(tu), fl_v = floorf(tv);
  const float bu = (float)geo.iu + fl_u, bv = (float)geo.iv + fl_v;  // texel indices (exact integers)
  const float wu = tu - fl_u, wv = tv - fl_v;
  if (!(bu + wu >= 0.0f && bv + wv >= 0.0f && bu + wu <= (float)(S.w - 1) && bv + wv <= (float)(S.h - 1)))
    return false;
  const float4 g = gather4<kMode == kSrcBf16 ? kSrcBf16 : kSrcExact>(S.tex, bu + 1.0f, bv + 1.0f);
  // gather order: (x0,y1) (x1,y1) (x1,y0) (x0,y0)
  const float p00 = g.w, p10 = g.z, p01 = g.x, p11 = g.y;
  const float top = fmaf(wu, p10 - p00, p00);
  const float bot = fmaf(wu, p11 - p01, p01);
  *s = fmaf(wv, bot - top, top);
  *r = __ldg(J.pref + (size_t)ry * J.w + rx);
  *mk = m;
  q[0] = h.qc[0] + dq0;
  q[1] = h.qc[1] + dq1;
  if (kGrad) {
    const float un = Y[0] * iz, vn = Y[1] * iz;
    const float gu = fmaf(wv, (p11 - p01) - (p10 - p00), p10 - p00);
    const float gv = bot - top;
    const float a = gu * S.fx * iz, c = gv * S.fy * iz;
    G[0] = a;
    G[1] = c;
    G[2] = -fmaf(a, un, c * vn);
  }
  return true;
}

template <int kMode>
__device__ ViewMom view_moments(const Job& J, const SrcView& S, const ViewGeo& geo, const AdjHyp& h) {
  ViewMom mo{};
  mo.valid = false;
  const int hw = J.patch_half;
  float X[3], Y[3], G[3], s, r, m, q[2];
  // the window centre must lie in front of the source camera
  if (!geo.ok) return mo;
  // shift: the window-centre samples (a source window whose centre is not
  // readable takes its first valid sample)
  float s0 = 0.f, r0 = 0.f;
  bool have0 = adj_sample<kMode, false>(J, S, geo, h, 0, 0, &s0, &r0, X, Y, G, &m, q);
  float n = 0.f, sr = 0.f, ss = 0.f, srr = 0.f, sss = 0.f, srs = 0.f;
  float cr = 0.f, cs = 0.f, crr = 0.f, css = 0.f, crs = 0.f;
  for (int dy = -hw; dy <= hw; ++dy) {
    float a_r = 0.f, a_s = 0.f, a_rr = 0.f, a_ss = 0.f, a_rs = 0.f;
    for (int dx = -hw; dx <= hw; ++dx) {
      if (!adj_sample<kMode, false>(J, S, geo, h, dx, dy, &s, &r, X, Y, G, &m, q)) continue;
      if (!have0) {
        s0 = s;
        r0 = r;
        have0 = true;
      }
      const float rv = r - r0, sv = s - s0;
      a_r += rv;
      a_s += sv;
      a_rr = fmaf(rv, rv, a_rr);
      a_ss = fmaf(sv, sv, a_ss);
      a_rs = fmaf(rv, sv, a_rs);
      n += 1.0f;
    }
    kahan_add(sr, cr, a_r);
    kahan_add(ss, cs, a_s);
    kahan_add(srr, crr, a_rr);
    kahan_add(sss, css, a_ss);
    kahan_add(srs, crs, a_rs);
  }
  if (n < (float)J.min_valid) return mo;
  const float inv_n = 1.0f / n;
  const float mr = sr * inv_n, ms = ss * inv_n;
  mo.n = n;
  mo.srr = srr - n * mr * mr;  // centred sums
  mo.sss = sss - n * ms * ms;
  mo.srs = srs - n * mr * ms;
  mo.mr = mr + r0;  // means of the unshifted values
  mo.ms = ms + s0;
  const float denom = sqrtf(mo.srr * mo.sss);
  if (!(denom >= 1e-9f * n)) return mo;
  mo.ncc = fminf(1.0f, fmaxf(-1.0f, mo.srs / denom));
  mo.valid = true;
  return mo;
}

// Second pass of one view: the gradient (3) and Gauss-Newton matrix (6, upper
// triangle) of c = 1 - NCC in the pixel parameters (d, theta, phi); with
// kPose also in the view's 6 pose parameters (gp, Hp 21).
template <int kMode, bool kPose>
__device__ void view_adjoint(const Job& J, const SrcView& S, const ViewGeo& geo, const AdjHyp& h, const ViewMom& mo,
                             float g[3], float H[6], float* gp, float* Hp) {
  const float* A = geo.A;
  const int hw = J.patch_half;
  float Sd[3] = {0, 0, 0}, Sdd[6] = {0, 0, 0, 0, 0, 0}, Ssd[3] = {0, 0, 0}, Sed[3] = {0, 0, 0};
  float Pd[6], Pdd[kPoseH], Psd[6], Ped[6];
  // residual weight: NCC sqrt(S_rr / S_ss)
  const float rho = mo.ncc * sqrtf(mo.srr / mo.sss);
  if (kPose) {
    for (int i = 0; i < 6; ++i) Pd[i] = Psd[i] = Ped[i] = 0.f;
    for (int i = 0; i < kPoseH; ++i) Pdd[i] = 0.f;
  }
  for (int dy = -hw; dy <= hw; ++dy) {
    for (int dx = -hw; dx <= hw; ++dx) {
      float X[3], Y[3], G[3], s, r, m, q[2];
      if (!adj_sample<kMode, true>(J, S, geo, h, dx, dy, &s, &r, X, Y, G, &m, q)) continue;
      const float st = s - mo.ms, rt = r - mo.mr;
      const float e = fmaf(rho, st, -rt);
      // w = A^T G = dI/dX
      float w[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) w[j] = fmaf(A[j], G[0], fmaf(A[3 + j], G[1], A[6 + j] * G[2]));
      const float qx = q[0], qy = q[1];  // the sample's ray (z = 1)
      const float wq = fmaf(w[0], qx, fmaf(w[1], qy, w[2]));
      const float dd = fmaf(w[0], X[0], fmaf(w[1], X[1], w[2] * X[2])) * h.id;
      const float im = rcp_approx(m);
      const float cn = wq * h.d * (im * im);
      float dn[3];
      dn[0] = cn * fmaf(h.qc[0], m, -h.kappa * qx);
      dn[1] = cn * fmaf(h.qc[1], m, -h.kappa * qy);
      dn[2] = cn * fmaf(h.qc[2], m, -h.kappa);
      const float dk[3] = {dd, fmaf(dn[0], h.nt[0], fmaf(dn[1], h.nt[1], dn[2] * h.nt[2])),
                           fmaf(dn[0], h.np[0], fmaf(dn[1], h.np[1], dn[2] * h.np[2]))};
      int t = 0;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        Sd[i] += dk[i];
        Ssd[i] = fmaf(st, dk[i], Ssd[i]);
        Sed[i] = fmaf(e, dk[i], Sed[i]);
#pragma unroll
        for (int j = i; j < 3; ++j, ++t) Sdd[t] = fmaf(dk[i], dk[j], Sdd[t]);
      }
      if (kPose) {
        // dI/dw = Y x G, dI/dtau = G
        const float pk[6] = {fmaf(Y[1], G[2], -Y[2] * G[1]), fmaf(Y[2], G[0], -Y[0] * G[2]),
                             fmaf(Y[0], G[1], -Y[1] * G[0]), G[0], G[1], G[2]};
        int u = 0;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          Pd[i] += pk[i];
          Psd[i] = fmaf(st, pk[i], Psd[i]);
          Ped[i] = fmaf(e, pk[i], Ped[i]);
#pragma unroll
          for (int j = i; j < 6; ++j, ++u) Pdd[u] = fmaf(pk[i], pk[j], Pdd[u]);
        }
      }
    }
  }
  const float inv_ss = 1.0f / mo.sss;
  const float inv_rs = rsqrtf(mo.srr * mo.sss);
  const float inv_n = 1.0f / mo.n;
  int t = 0;
  for (int i = 0; i < 3; ++i) {
    g[i] = inv_rs * Sed[i];
    for (int j = i; j < 3; ++j, ++t)
      H[t] = inv_ss * (Sdd[t] - Sd[i] * Sd[j] * inv_n - Ssd[i] * Ssd[j] * inv_ss);
  }
  if (kPose) {
    int u = 0;
    for (int i = 0; i < 6; ++i) {
      gp[i] = inv_rs * Ped[i];
      for (int j = i; j < 6; ++j, ++u)
        Hp[u] = inv_ss * (Pdd[u] - Pd[i] * Pd[j] * inv_n - Psd[i] * Psd[j] * inv_ss);
    }
  }
}

// Builds the hypothesis; false when the plane does not face the camera at
// this pixel (the search's own rule).
__device__ __forceinline__ bool make_adj_hyp(const Job& J, int x, int y, float d, float theta, float phi,
                                             AdjHyp* h) {
  h->x = x;
  h->y = y;
  h->d = d;
  h->id = 1.0f / d;
  h->irfx = 1.0f / J.rfx;
  h->irfy = 1.0f / J.rfy;
  sph_normal(theta, phi, h->n, h->nt, h->np);
  h->qc[0] = ((float)x + 0.5f - J.rcx) / J.rfx;
  h->qc[1] = ((float)y + 0.5f - J.rcy) / J.rfy;
  h->qc[2] = 1.0f;
  h->kappa = h->n[0] * h->qc[0] + h->n[1] * h->qc[1] + h->n[2];
  const float rn = sqrtf(h->qc[0] * h->qc[0] + h->qc[1] * h->qc[1] + 1.0f);
  return d > 0.0f && h->kappa < -0.05f * rn;
}

// The aggregated cost (mean of the best_k view costs, the search's rule),
// its gradient in (d, theta, phi), its Gauss-Newton matrix, and -- when
// pose_grad is non-null -- the gradient in every source's pose (zero for
// views outside the best_k).  Returns the number of views averaged (0 =
// invalid hypothesis).
template <int kMode>
__device__ int plane_adjoint(const Job& J, const AdjHyp& h, float* cost, float g[3], float H[6], float* pose_grad) {
  float vc[kMaxSources];
  ViewMom mom[kMaxSources];
  int nvalid = 0;
  const int ns = min(J.num_src, kMaxSources);
  for (int s = 0; s < ns; ++s) {
    const ViewGeo geo = view_geo(J, J.src[s], h);
    mom[s] = view_moments<kMode>(J, J.src[s], geo, h);
    vc[s] = mom[s].valid ? 1.0f - mom[s].ncc : kCostInf;
    nvalid += mom[s].valid;
  }
  for (int i = 0; i < 3; ++i) g[i] = 0.f;
  for (int i = 0; i < 6; ++i) H[i] = 0.f;
  if (pose_grad)
    for (int i = 0; i < 6 * ns; ++i) pose_grad[i] = 0.f;
  *cost = kCostInf;
  if (nvalid == 0) return 0;
  const int k = (J.best_k <= 0 || J.best_k >= nvalid || J.best_k > kMaxBestK) ? nvalid : J.best_k;
  // select the k lowest costs, ties to the lower source index
  bool sel[kMaxSources];
  for (int s = 0; s < ns; ++s) sel[s] = false;
  float csum = 0.f;
  for (int t = 0; t < k; ++t) {
    int best = -1;
    for (int s = 0; s < ns; ++s)
      if (mom[s].valid && !sel[s] && (best < 0 || vc[s] < vc[best])) best = s;
    sel[best] = true;
    csum += vc[best];
  }
  const float inv_k = 1.0f / (float)k;
  *cost = csum * inv_k;
  for (int s = 0; s < ns; ++s) {
    if (!sel[s]) continue;
    float gs[3], Hs[6], gp[6], Hp[kPoseH];
    const ViewGeo geo = view_geo(J, J.src[s], h);
    if (pose_grad)
      view_adjoint<kMode, true>(J, J.src[s], geo, h, mom[s], gs, Hs, gp, Hp);
    else
      view_adjoint<kMode, false>(J, J.src[s], geo, h, mom[s], gs, Hs, gp, Hp);
    for (int i = 0; i < 3; ++i) g[i] += gs[i] * inv_k;
    for (int i = 0; i < 6; ++i) H[i] += Hs[i] * inv_k;
    if (pose_grad)
      for (int i = 0; i < 6; ++i) pose_grad[6 * s + i] = gp[i] * inv_k;
  }
  return k;
}

// Solves (H + lambda diag(H)) x = -g for the symmetric 3 x 3 H (upper
// triangle 00 01 02 11 12 22); false when singular.
__device__ __forceinline__ bool solve_lm3(const float H[6], const float g[3], float lambda, float x[3]) {
  const float a = H[0] * (1.0f + lambda), b = H[1], c = H[2];
  const float d = H[3] * (1.0f + lambda), e = H[4], f = H[5] * (1.0f + lambda);
  const float c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
  const float det = a * c00 + b * c01 + c * c02;
  if (!(fabsf(det) > 1e-30f)) return false;
  const float c11 = a * f - c * c, c12 = b * c - a * e, c22 = a * d - b * b;
  const float id = 1.0f / det;
  x[0] = -(c00 * g[0] + c01 * g[1] + c02 * g[2]) * id;
  x[1] = -(c01 * g[0] + c11 * g[1] + c12 * g[2]) * id;
  x[2] = -(c02 * g[0] + c12 * g[1] + c22 * g[2]) * id;
  return isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]);
}

}  // namespace rmvs
