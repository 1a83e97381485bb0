// pm.cu -- PatchMatch kernels: hypothesis evaluation, plane-mode red-black
// sweeps, compat-mode (reference) Jacobi sweeps, outputs, refinement.
//
// Plane mode (the GB300 engine): per-pixel plane hypotheses (inverse depth,
// normal), red-black checkerboard propagation -- a half-sweep updates one
// colour reading only the other colour, so it is race-free and
// deterministic -- with adaptive neighbour selection (best cost in each of 8
// regions) and random perturbation; cost = mean of the best_k view costs.
// Work that cannot change a pixel's fate is skipped (a propagation candidate
// equal to the one just rejected; the remaining source windows of a
// candidate once its best-k bound rules it out): the maps do not depend on
// it, and Job::prune = 0 turns it off.
//
// Compat mode (drop-in parity): the reference PatchMatchStereo exactly --
// fronto-parallel inverse-depth hypotheses, translated windows, and the
// reference's Jacobi sweeps (every pixel reads the sweep's snapshot,
// patchmatch_stereo.cpp:615-740), run one thread per pixel; the reference's
// row-block xorshift draws are generated on the host in its scan order.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdio>
#include <type_traits>

#include "adjoint.cuh"
#include "cost.cuh"
#include "kernels.h"

namespace rmvs {

// ---------------------------------------------------------------------------
// per-thread source-ray cache in shared memory: P[s][c] as float2 (hi, lo)
// ---------------------------------------------------------------------------
struct PCache {
  float2* base;
  int stride;  // threads per block
  int tid;
  __device__ __forceinline__ void get(int s, ff P[3]) const {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 v = base[(s * 3 + c) * stride + tid];
      P[c] = ff{v.x, v.y};
    }
  }
  __device__ __forceinline__ void put(int s, const ff P[3]) const {
#pragma unroll
    for (int c = 0; c < 3; ++c) base[(s * 3 + c) * stride + tid] = make_float2(P[c].hi, P[c].lo);
  }
};

__device__ __forceinline__ void fill_pcache(const Job& J, const PCache& pc, int x, int y, float* rx, float* ry) {
  if (J.hyp && !J.ref_distorted) {
    // plane mode, pinhole reference: the pixel ray and P_s = A_s ray in
    // float-float (~44-bit mantissa) -- no FP64 on the device, whose rate on
    // this part is 1/64 of FP32
    const ff xr = ff_div(ff_add(ff_make((float)x + 0.5f), ff{-J.ffrcx.hi, -J.ffrcx.lo}), J.ffrx);
    const ff yr = ff_div(ff_add(ff_make((float)y + 0.5f), ff{-J.ffrcy.hi, -J.ffrcy.lo}), J.ffry);
    for (int s = 0; s < J.num_src; ++s) {
      const SrcView& S = J.src[s];
      ff P[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) P[i] = ff_add(ff_add(ff_mul(S.Aff[3 * i], xr), ff_mul(S.Aff[3 * i + 1], yr)), S.Aff[3 * i + 2]);
      pc.put(s, P);
    }
    *rx = __fadd_rn(xr.hi, xr.lo);
    *ry = __fadd_rn(yr.hi, yr.lo);
    return;
  }
  double ray[3];
  ref_ray(J, x + 0.5, y + 0.5, ray);
  for (int s = 0; s < J.num_src; ++s) {
    ff P[3];
    source_rays(J, J.src[s], ray, P);
    pc.put(s, P);
  }
  *rx = (float)ray[0];
  *ry = (float)ray[1];
}

// ---------------------------------------------------------------------------
// full hypothesis evaluation over all sources
// ---------------------------------------------------------------------------
struct HypCost {
  float cost;
  int support;
};

__device__ __forceinline__ HypCost finish_plane(float* best, float sum_all, int nvalid, int best_k,
                                                float photo_threshold) {
  HypCost r{kCostInf, nvalid};
  if (nvalid == 0) return r;
  float c;
  if (best_k <= 0 || best_k >= nvalid || best_k > kMaxBestK) {
    c = sum_all / (float)nvalid;
  } else {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kMaxBestK; ++i)
      if (i < best_k) s += best[i];
    c = s / (float)best_k;
  }
  if (c > 3.0f * photo_threshold) c = kCostInf;
  r.cost = c;
  return r;
}

// The cost of one plane hypothesis from its views: view(s, active) evaluates
// source view s and returns its NCC (valid = -1: not sampled); the cost is
// the mean of the best_k view costs 1 - NCC.  Exact pruning: view costs lie
// in [0, 2], so after each view the final cost is bounded below by letting
// every remaining view be valid at cost 0 -- with K = best_k (or all views),
// n valid so far, r views left and k' = min(K, n + r), cost >= (sum of the
// k' - r lowest costs so far) / k'.  Once that bound is above `beat` (the
// cost a candidate must get below to be taken, with a relative margin that
// covers the rounding of both sums) the remaining views cannot change the
// decision and are not evaluated: the candidate is returned as rejected.
// kCollective: view() is called for every view whatever this lane's state
// (the staged schedule's views are warp-collective), `active` telling it
// whether this lane's hypothesis still needs the view.
template <bool kCollective, class ViewFn>
__device__ __forceinline__ HypCost plane_hyp_cost(const Job& J, bool live, const ViewFn& view, float* view_cost,
                                                  int* counts, float beat) {
  float best[kMaxBestK];
#pragma unroll
  for (int i = 0; i < kMaxBestK; ++i) best[i] = kCostInf;
  float sum_all = 0.f;
  int nvalid = 0;
  const bool all_views = J.best_k <= 0 || J.best_k > kMaxBestK;
  const int K = all_views ? J.num_src : J.best_k;
  const float bar = beat * (1.0f + 4e-6f);
  bool pruned = false;
  for (int s = 0; s < J.num_src; ++s) {
    ViewResult v{0.0f, -1};  // skipped: not sampled
    if (kCollective)
      v = view(s, live && !pruned);
    else if (!pruned)
      v = view(s, true);
    if (counts) counts[1] += v.valid >= 0;
    float c = kCostInf;
    if (v.valid > 0) {
      c = 1.0f - v.ncc;
      ++nvalid;
      sum_all += c;
#pragma unroll
      for (int i = 0; i < kMaxBestK; ++i) {
        const float lo = fminf(best[i], c), hi = fmaxf(best[i], c);
        best[i] = lo;
        c = hi;
      }
      c = 1.0f - v.ncc;
    }
    if (view_cost) view_cost[s] = c;
    const int left = J.num_src - 1 - s;
    if (left > 0 && left < K && nvalid > 0) {
      const int kk = min(K, nvalid + left), j = kk - left;
      float lb;
      if (all_views) {
        lb = sum_all;  // j == nvalid: every valid view so far
      } else {
        lb = 0.f;
#pragma unroll
        for (int i = 0; i < kMaxBestK; ++i)
          if (i < j) lb += best[i];
      }
      pruned = pruned || (j > 0 && lb > bar * (float)kk);
    }
  }
  if (!live || pruned) return HypCost{kCostInf, 0};
  return finish_plane(best, sum_all, nvalid, J.best_k, J.photo_threshold);
}

template <int H, int kMode, class Ref>
__device__ HypCost eval_plane_hyp(const Job& J, const PCache& pc, int x, int y, float rx, float ry, float rho,
                                  float nx, float ny, float nz, const RefWindow& rw, const Ref& ref, float* view_cost,
                                  int* counts = nullptr, float beat = kCostInf) {
  HypCost bad{kCostInf, 0};
  PlaneHyp hp;
  if (!(rho > 0.0f) || rho < J.rho_min || rho > J.rho_max || !make_plane_hyp(J, rx, ry, rho, nx, ny, nz, &hp)) {
    if (view_cost)
      for (int s = 0; s < J.num_src; ++s) view_cost[s] = kCostInf;
    return bad;
  }
  if (counts) ++counts[0];
  return plane_hyp_cost<false>(
      J, true,
      [&](int s, bool) {
        ff P[3];
        pc.get(s, P);
        return eval_view_plane<H, kMode>(J, J.src[s], x, y, P, hp, rw, ref);
      },
      view_cost, counts, beat);
}

// COMPAT: 1 - mean NCC over valid views (patchmatch_stereo.cpp:344-418).
__device__ HypCost eval_compat_hyp(const Job& J, const PCache& pc, int x, int y, double inv, const RefWindow& rw,
                                   float* view_cost) {
  HypCost bad{kCostInf, 0};
  if (inv <= 1e-9) return bad;
  const double depth = 1.0 / inv;
  if (depth < J.min_depth || depth > J.max_depth) return bad;
  const float hi = (float)inv;
  const ff rho{hi, (float)(inv - (double)hi)};
  float sum = 0.f;
  int nvalid = 0;
  for (int s = 0; s < J.num_src; ++s) {
    ff P[3];
    pc.get(s, P);
    const ViewResult v = eval_view_compat(J, J.src[s], x, y, P, rho, hi, rw);
    if (v.valid) {
      ++nvalid;
      sum += v.ncc;
    }
    if (view_cost) view_cost[s] = v.valid ? 1.0f - v.ncc : kCostInf;
  }
  HypCost r{kCostInf, nvalid};
  if (nvalid == 0) return r;
  float c = 1.0f - sum / (float)nvalid;
  if (c > 3.0f * J.photo_threshold) c = kCostInf;
  r.cost = c;
  return r;
}

// ---------------------------------------------------------------------------
// batch evaluation of given hypotheses (parity instrument, adjoint driver)
// ---------------------------------------------------------------------------
template <int H, int kMode>
__global__ void __launch_bounds__(128, 4) k_eval_hyps(Job J, int mode, int n, const int* __restrict__ px, const int* __restrict__ py,
                            const double* __restrict__ inv, const float* __restrict__ normals, float* out_cost,
                            int* out_support, float* out_view_cost) {
  extern __shared__ float2 smem[];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  PCache pc{smem, (int)blockDim.x, (int)threadIdx.x};
  if (i >= n) return;
  const int x = px[i], y = py[i];
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  float* vc = out_view_cost ? out_view_cost + (size_t)i * J.num_src : nullptr;
  HypCost r;
  if (mode == 0) {
    const RefWindow rw = ref_window(J, x, y, true);
    r = eval_compat_hyp(J, pc, x, y, inv[i], rw, vc);
  } else {
    const RefWindow rw = ref_window(J, x, y, J.half_pixel);
    const GlobalRef ref{J.pref, J.w, x, y};
    r = eval_plane_hyp<H, kMode>(J, pc, x, y, rx, ry, (float)inv[i], normals[3 * i], normals[3 * i + 1], normals[3 * i + 2],
                          rw, ref, vc);
  }
  out_cost[i] = r.cost;
  out_support[i] = r.support;
}

// ---------------------------------------------------------------------------
// plane mode
// ---------------------------------------------------------------------------
__device__ __forceinline__ void random_normal(Rng& g, float rx, float ry, float* nx, float* ny, float* nz) {
  // uniform direction, flipped to face the camera, kept off grazing angles
  const float rn = rsqrtf(rx * rx + ry * ry + 1.0f);
  for (int t = 0; t < 8; ++t) {
    const float z = g.sym();
    const float phi = 6.28318530718f * g.uniform();
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float a = r * __cosf(phi), b = r * __sinf(phi), c = z;
    float d = (a * rx + b * ry + c) * rn;
    if (d > 0.f) {
      a = -a;
      b = -b;
      c = -c;
      d = -d;
    }
    if (d < -0.2f) {
      *nx = a;
      *ny = b;
      *nz = c;
      return;
    }
  }
  *nx = 0.f;
  *ny = 0.f;
  *nz = -1.f;
}

__device__ __forceinline__ void perturb_normal(Rng& g, float rx, float ry, float scale, float* nx, float* ny,
                                               float* nz) {
  float a = *nx + scale * g.sym(), b = *ny + scale * g.sym(), c = *nz + scale * g.sym();
  const float inv = rsqrtf(a * a + b * b + c * c);
  a *= inv;
  b *= inv;
  c *= inv;
  const float rn = rsqrtf(rx * rx + ry * ry + 1.0f);
  if ((a * rx + b * ry + c) * rn < -0.2f) {
    *nx = a;
    *ny = b;
    *nz = c;
  }
}

__device__ __forceinline__ Rng pixel_rng(const Job& J, int idx, int iter, int salt) {
  Rng g;
  g.s = mix64(J.seed ^ ((uint64_t)idx * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)(iter + 1) << 40) ^
              ((uint64_t)salt << 56));
  return g;
}

// ---------------------------------------------------------------------------
// batched plane kernels
// ---------------------------------------------------------------------------
// Every plane-mode run goes through these kernels.  A batch is any set of up
// to kBatchJobs reference views -- uneven sizes and source counts -- that
// share the window size and the interpolation mode.  The batch's job records
// travel in the kernel-parameter (constant) bank: a block reads the record of
// its job with uniform constant loads, which the compiler can re-issue instead
// of holding every field in registers (a copy in shared memory costs the
// unrolled window code hundreds of bytes of spills).  Work items are tiles;
// B.start holds the exclusive prefix of the jobs' tile counts, so an item
// finds its job by a binary search.
__device__ __forceinline__ int find_job(const PlaneBatch& B, int item) {
  int lo = 0, hi = B.njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (B.start[mid] <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Pixel-tile kernels (init, refine, output): one 32 x 4 block per 32 x 4
// pixel tile, grid = the batch's tile count.  Returns the block's job and
// whether this thread's pixel lies inside its image.
__device__ __forceinline__ bool pixel_item(const PlaneBatch& B, int* job, int* x, int* y) {
  const int j = find_job(B, (int)blockIdx.x);
  const int local = (int)blockIdx.x - B.start[j];
  const int tx = (B.jobs[j].w + 31) >> 5;
  *job = j;
  *x = (local % tx) * 32 + (int)threadIdx.x;
  *y = (local / tx) * 4 + (int)threadIdx.y;
  return *x < B.jobs[j].w && *y < B.jobs[j].h;
}

// A neighbour's plane {rho_n at its ray (rxn, ryn), n} carried to the ray
// (rx, ry): the inverse depth at which that ray meets the plane, or -1 when
// the plane does not face the camera along either ray.
__device__ __forceinline__ void plane_candidate_transfer(const float4 hn, float rxn, float ryn, float rx, float ry,
                                                         float* rho) {
  // the neighbour's plane n . X = kappa_n / rho_n, evaluated on this pixel's ray
  const float kn = hn.y * rxn + hn.z * ryn + hn.w;
  const float kp = hn.y * rx + hn.z * ry + hn.w;
  *rho = (kn < 0.f && kp < 0.f) ? hn.x * kp / kn : -1.0f;
}

// Random initialisation (and seed cells) + initial cost.  Block 0 also zeroes
// the work counters of the persistent sweeps that follow, and each job's
// first pixel zeroes its filled counter.
template <int H, int kMode>
__global__ void __launch_bounds__(128, 4) k_plane_init(const __grid_constant__ PlaneBatch B, int* queues,
                                                       int num_queues) {
  extern __shared__ float2 smem[];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  if (blockIdx.x == 0)
    for (int q = tid; q < num_queues; q += 128) queues[q] = 0;
  int j, x, y;
  if (!pixel_item(B, &j, &x, &y)) return;
  const Job& J = B.jobs[j];
  PCache pc{smem, 128, tid};
  const int idx = y * J.w + x;
  if (idx == 0) *J.out_filled = 0u;
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  Rng g = pixel_rng(J, idx, -1, 1);
  float rho = J.rho_min + (J.rho_max - J.rho_min) * g.uniform();
  float nx, ny, nz;
  random_normal(g, rx, ry, &nx, &ny, &nz);
  if (J.coarse_hyp) {
    // the parent's plane at the half-resolution level, carried to this ray
    const int px = min(x >> 1, J.coarse_w - 1), py = min(y >> 1, J.coarse_h - 1);
    const int pi = py * J.coarse_w + px;
    if (J.coarse_cost[pi] < kCostInf) {
      const float4 hn = J.coarse_hyp[pi];
      float rt;
      plane_candidate_transfer(hn, ((float)px + 0.5f - J.crcx) / J.crfx, ((float)py + 0.5f - J.crcy) / J.crfy, rx,
                               ry, &rt);
      if (rt >= J.rho_min && rt <= J.rho_max) {
        rho = rt;
        nx = hn.y;
        ny = hn.z;
        nz = hn.w;
      }
    }
  }
  if (J.seed_depth) {
    const int cx = min(x / 32, J.seed_gx - 1);
    const int cy = y / 32;
    const float sd = J.seed_depth[cy * J.seed_gx + cx];
    if (sd > 0.f) {
      rho = 1.0f / sd;
      nx = 0.f;
      ny = 0.f;
      nz = -1.f;
    }
  }
  const RefWindow rw = ref_window(J, x, y, J.half_pixel);
  const GlobalRef ref{J.pref, J.w, x, y};
  const HypCost c = eval_plane_hyp<H, kMode>(J, pc, x, y, rx, ry, rho, nx, ny, nz, rw, ref, nullptr);
  J.hyp[idx] = make_float4(rho, nx, ny, nz);
  J.cost[idx] = c.cost;
  J.support[idx] = (uint8_t)min(c.support, 255);
}

// Propagation skips a candidate that is the pixel's current plane: same
// normal bits and an inverse depth within this relative distance (the FP32
// plane transfer through a chain of neighbours rounds at ~1e-7 per step).
constexpr float kSamePlaneRel = 4e-6f;

// Adaptive checkerboard regions (other-colour pixels only: dx + dy odd).
// 4 near "V" regions of 7 pixels and 4 far strips of 11 pixels.
__constant__ signed char c_near[4][7][2] = {
    {{0, -1}, {-1, -2}, {1, -2}, {-2, -3}, {2, -3}, {-3, -4}, {3, -4}},
    {{0, 1}, {-1, 2}, {1, 2}, {-2, 3}, {2, 3}, {-3, 4}, {3, 4}},
    {{-1, 0}, {-2, -1}, {-2, 1}, {-3, -2}, {-3, 2}, {-4, -3}, {-4, 3}},
    {{1, 0}, {2, -1}, {2, 1}, {3, -2}, {3, 2}, {4, -3}, {4, 3}}};


// Reference-window statistics from the shared tile (same values as
// ref_window for pixels whose window lies inside the image).
template <int H>
__device__ __forceinline__ RefWindow tile_window(const Job& J, const TileRef& t, int x, int y) {
  RefWindow rw;
  rw.full = x >= H && y >= H && x + H <= J.w - 1 - J.half_pixel && y + H <= J.h - 1 - J.half_pixel;
  if (!rw.full) return ref_window(J, x, y, J.half_pixel);
  float s = 0.f;
#pragma unroll 1
  for (int dy = -H; dy <= H; ++dy) {
    const TileRow r = t.row<H>(dy);
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) s += (k & 1) ? r.odd(k >> 1) : r.even(k >> 1);
  }
  rw.mean = s / (float)((2 * H + 1) * (2 * H + 1));
  float q = 0.f;
#pragma unroll 1
  for (int dy = -H; dy <= H; ++dy) {
    const TileRow r = t.row<H>(dy);
    float qr = 0.f;
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) {
      const float d = ((k & 1) ? r.odd(k >> 1) : r.even(k >> 1)) - rw.mean;
      qr = fmaf(d, d, qr);
    }
    q += qr;
  }
  rw.sxx = q;
  return rw;
}

// Propagation candidate of region r (0-7) for pixel (x, y): the plane of the
// region's lowest-cost neighbour, carried to this pixel's ray.  False when the
// region offers nothing to learn: no neighbour with a finite cost, the
// current plane again (same normal, inverse depth within rounding of the
// transfer -- in a converged region most regions propose exactly this), or,
// with pruning, the previous region's candidate again (the same plane reached
// through another neighbour: it was rejected, and its cost has not changed).
__device__ __forceinline__ bool propagation_candidate(const Job& J, int x, int y, int r, float rx, float ry,
                                                      float ifx, float ify, const float4& cur, float4& last,
                                                      float4* cand) {
  int best_n = -1;
  float best_c = kCostInf;
  if (r < 4) {
    for (int k = 0; k < 7; ++k) {
      const int nx_ = x + c_near[r][k][0], ny_ = y + c_near[r][k][1];
      if (nx_ < 0 || ny_ < 0 || nx_ >= J.w || ny_ >= J.h) continue;
      const float c = J.cost[ny_ * J.w + nx_];
      if (c < best_c) {
        best_c = c;
        best_n = ny_ * J.w + nx_;
      }
    }
  } else {
    const int d = r - 4;
    const int sx = d == 2 ? -1 : (d == 3 ? 1 : 0);
    const int sy = d == 0 ? -1 : (d == 1 ? 1 : 0);
    for (int k = 0; k < 11; ++k) {
      const int off = 3 + 2 * k;
      const int nx_ = x + sx * off, ny_ = y + sy * off;
      if (nx_ < 0 || ny_ < 0 || nx_ >= J.w || ny_ >= J.h) continue;
      const float c = J.cost[ny_ * J.w + nx_];
      if (c < best_c) {
        best_c = c;
        best_n = ny_ * J.w + nx_;
      }
    }
  }
  if (best_n < 0 || best_c >= kCostInf) return false;
  const float4 hn = J.hyp[best_n];
  const int nxp = best_n % J.w, nyp = best_n / J.w;
  float rho;
  plane_candidate_transfer(hn, ((float)nxp + 0.5f - J.rcx) * ifx, ((float)nyp + 0.5f - J.rcy) * ify, rx, ry, &rho);
  if (!(rho > 0.f)) return false;
  if (hn.y == cur.y && hn.z == cur.z && hn.w == cur.w && fabsf(rho - cur.x) <= kSamePlaneRel * cur.x) return false;
  if (J.prune && hn.y == last.y && hn.z == last.z && hn.w == last.w && rho == last.x) return false;
  last = make_float4(rho, hn.y, hn.z, hn.w);
  *cand = last;
  return true;
}

// Refinement candidate k (0-4) around the current plane `cur`: a random
// plane (k = 0), the inverse depth perturbed (k = 1), the normal perturbed
// (k = 2), both (k = 3) -- ranges shrinking by half per iteration (`scale`)
// -- and the current depth on a fronto-parallel plane (k = 4, the reference's
// model; false when the plane already is one).  The draws are made whether
// or not the candidate is then evaluated (exploring()), so the random stream
// of every pixel is the same under any exploration schedule.
__device__ __forceinline__ bool refinement_candidate(const Job& J, Rng& g, int k, const float4& cur, float rx,
                                                     float ry, float scale, float span, float4* cand) {
  float rho = cur.x, nx = cur.y, ny = cur.z, nz = cur.w;
  if (k == 0) {
    rho = J.rho_min + span * g.uniform();
    random_normal(g, rx, ry, &nx, &ny, &nz);
  } else if (k == 4) {
    if (nx == 0.f && ny == 0.f) return false;
    nx = 0.f;
    ny = 0.f;
    nz = -1.f;
  } else {
    if (k & 1) rho = cur.x + 0.25f * span * scale * g.sym();
    if (k & 2) perturb_normal(g, rx, ry, 0.5f * scale, &nx, &ny, &nz);
  }
  *cand = make_float4(rho, nx, ny, nz);
  return true;
}

// Whether iteration `iter` evaluates refinement candidate k: the exploration
// candidates (k = 0, the random plane; k = 4, the fronto-parallel plane) stop
// at the job's explore_iters -- by then the search has converged and they
// almost never win (at 1920x1440 after coarse-to-fine initialisation: the
// random plane 0.04-0.4 % of its evaluations, the fronto-parallel plane
// 0.2-2.4 %) -- while propagation and the local perturbations go on.
__device__ __forceinline__ bool exploring(const Job& J, int k, int iter) {
  return (k != 0 && k != 4) || J.explore_iters <= 0 || iter < J.explore_iters;
}

// The evaluation counters of a warp into the job's counter (one atomic per
// warp and counter).
__device__ __forceinline__ void add_counts(const Job& J, unsigned int mask, const int* counts, int n) {
  for (int i = 0; i < n; ++i) {
    const unsigned int v = __reduce_add_sync(mask, (unsigned int)counts[i]);
    if ((threadIdx.x & 31) == (__ffs(mask) - 1) && v) atomicAdd(J.eval_counter + i, (unsigned long long)v);
  }
}

// One red-black half-sweep of one pixel: propagation from the best-cost
// neighbour of each of the 8 adaptive regions, then 5 refinement hypotheses.
template <int H, int kMode, class RefT>
__device__ __forceinline__ void sweep_pixel(const Job& J, const PCache& pc, const RefT& ref, const RefWindow& rw,
                                            int x, int y, int color, int iter) {
  const int idx = y * J.w + x;
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  float4 cur = J.hyp[idx];
  float cur_cost = J.cost[idx];
  int cur_sup = J.support[idx];
  const float ifx = 1.0f / J.rfx, ify = 1.0f / J.rfy;
  int counts[2] = {0, 0};  // hypotheses, source windows sampled

  float4 last = make_float4(-1.f, 0.f, 0.f, 0.f);  // the last candidate evaluated
  for (int r = 0; r < 8; ++r) {
    float4 cand;
    if (!propagation_candidate(J, x, y, r, rx, ry, ifx, ify, cur, last, &cand)) continue;
    const HypCost c = eval_plane_hyp<H, kMode>(J, pc, x, y, rx, ry, cand.x, cand.y, cand.z, cand.w, rw, ref, nullptr,
                                               counts, J.prune ? cur_cost : kCostInf);
    if (c.cost < cur_cost) {
      cur_cost = c.cost;
      cur = cand;
      cur_sup = c.support;
    }
  }
  Rng g = pixel_rng(J, idx, iter, 2 + color);
  const float scale = exp2f(-(float)iter);  // 1, 1/2, 1/4, ...
  const float span = J.rho_max - J.rho_min;
  for (int k = 0; k < 5; ++k) {
    float4 cand;
    if (!refinement_candidate(J, g, k, cur, rx, ry, scale, span, &cand) || !exploring(J, k, iter)) continue;
    const HypCost c = eval_plane_hyp<H, kMode>(J, pc, x, y, rx, ry, cand.x, cand.y, cand.z, cand.w, rw, ref, nullptr,
                                               counts, J.prune ? cur_cost : kCostInf);
    if (c.cost < cur_cost) {
      cur_cost = c.cost;
      cur = cand;
      cur_sup = c.support;
    }
  }
  if (J.eval_counter) add_counts(J, __activemask(), counts, 2);
  J.hyp[idx] = cur;
  J.cost[idx] = cur_cost;
  J.support[idx] = (uint8_t)min(cur_sup, 255);
}

// ---- TMA staging of the reference tile ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The 3-D box {x, y, z} of `map` into shared memory, completion signalled
// on `bar` (expecting `bytes`).  x is a multiple of 8 floats (32 bytes), y
// may be negative or past the end: TMA fills zeros there.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar,
                                            uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// Waits for phase `parity` of `bar`, giving up after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

constexpr int kTmaWaitPolls = 1 << 22;

// ---- the staged-window schedule ----
// The 2-D box {x, y} of `map` (a tensor map in global memory) into shared
// memory, completion signalled on `bar`.  x is even (8-byte elements:
// 16-byte aligned rows); x or y may be negative or past the end (zeros).
__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, int x, int y, uint64_t* bar,
                                            uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// One warp's source box and its copy state (the same in every lane).
struct WarpBox {
  float2* box;     // kStageH rows x kStageW texel pairs, 128-byte aligned
  uint64_t* bar;   // the box's mbarrier (arrival count 1)
  uint32_t phase;  // parity of the next copy's completion
  int polls;       // wait limit
  int* err;        // set when a wait runs out
  bool dead;       // a wait ran out: no further copies into this box in this launch
};

// One source view of one candidate for the whole warp (every lane calls it;
// `act`: this lane's hypothesis is live for the view).  The lanes whose
// windows lie fully inside the source (the fast path) pool the texels they
// read -- the corners' footprints with a margin of one texel for rounding --
// into one box; when it fits kStageW x kStageH, lane 0 copies it from the
// view's pair image by TMA and every lane waits (bounded) for it, then those
// windows are read from shared memory.  Other windows, and full ones whose
// box does not fit, read the texture.  Either way a window's NCC is the same
// bit for bit.
template <int H, class Ref>
__device__ __forceinline__ ViewResult eval_view_staged(const Job& J, const SrcView& S, int x, int y, const ff P[3],
                                                       const PlaneHyp& hp, bool act, const RefWindow& rw,
                                                       const Ref& ref, WarpBox& wb, int* counts) {
  WindowPlace g;
  const bool geo = act && place_window<H>(J, S, P, hp, rw, &g);
  int x0 = 0x7fffffff, x1 = (int)0x80000000, y0 = 0x7fffffff, y1 = (int)0x80000000;
  if (geo && g.full) {
    // footprints of index coordinates in [min, max]: texels floor(min) - 1 ..
    // floor(max) + 1 (an exact tie reads one texel lower), plus the margin
    x0 = g.iu + (int)floorf(g.umin) - 2;
    x1 = g.iu + (int)floorf(g.umax) + 2;
    y0 = g.iv + (int)floorf(g.vmin) - 2;
    y1 = g.iv + (int)floorf(g.vmax) + 2;
  }
  x0 = __reduce_min_sync(0xffffffffu, x0);
  x1 = __reduce_max_sync(0xffffffffu, x1);
  y0 = __reduce_min_sync(0xffffffffu, y0);
  y1 = __reduce_max_sync(0xffffffffu, y1);
  const int ax = x0 & ~1;  // an even first pair: 16-byte TMA rows
  // pair element e of a box row holds texels ax + e and ax + e + 1, so the
  // texels ax .. x1 need x1 - ax <= kStageW; rows y0 .. y1 need kStageH
  bool staged = S.pair_map != nullptr && !wb.dead && x0 <= x1 && x1 - ax <= kStageW && y1 - y0 < kStageH;
  if (staged) {
    if ((threadIdx.x & 31) == 0) tma_load_2d(wb.box, S.pair_map, ax, y0, wb.bar, (uint32_t)kStageBytes);
    const bool ok = __all_sync(0xffffffffu, mbar_wait(wb.bar, wb.phase, wb.polls));
    wb.phase ^= 1u;
    if (!ok) {
      // the copy may still land: the box is not used again in this launch
      wb.dead = true;
      staged = false;
      if ((threadIdx.x & 31) == 0) atomicExch(wb.err, 1);
    }
  }
  ViewResult v{0.0f, -1};
  if (geo) {
    if (staged && g.full) {
      v = eval_view_box<H>(J, g, rw, ref, wb.box, ax, y0);
      ++counts[2];
    } else {
      v = eval_view_placed<H, kSrcExact>(J, S, x, y, g, hp, rw, ref);
    }
  }
  __syncwarp();  // every lane is done with the box before the next copy into it
  return v;
}

// eval_plane_hyp for the staged schedule: the view loop runs in step across
// the warp (J is the same for the whole block); `have` = this lane has a
// candidate in this slot.
template <int H, class Ref>
__device__ __forceinline__ HypCost eval_plane_hyp_staged(const Job& J, const PCache& pc, int x, int y, float rx,
                                                         float ry, const float4& cand, bool have, const RefWindow& rw,
                                                         const Ref& ref, int* counts, float beat, WarpBox& wb) {
  PlaneHyp hp;
  const float rho = cand.x;
  const bool live = have && rho > 0.0f && !(rho < J.rho_min) && !(rho > J.rho_max) &&
                    make_plane_hyp(J, rx, ry, rho, cand.y, cand.z, cand.w, &hp);
  if (live) ++counts[0];
  return plane_hyp_cost<true>(
      J, live,
      [&](int s, bool act) {
        ff P[3] = {};
        if (act) pc.get(s, P);
        return eval_view_staged<H>(J, J.src[s], x, y, P, hp, act, rw, ref, wb, counts);
      },
      nullptr, counts, beat);
}

// sweep_pixel for the staged schedule: every lane of the warp runs every
// candidate slot and view in step; a lane outside the image, or without a
// candidate in a slot, only takes part in the warp's collective steps.
template <int H, class RefT>
__device__ __forceinline__ void sweep_pixel_staged(const Job& J, const PCache& pc, const RefT& ref, bool inside,
                                                   int x, int y, int color, int iter, WarpBox& wb) {
  const int idx = inside ? y * J.w + x : 0;
  RefWindow rw{0.0f, 0.0f, false};
  float rx = 0.f, ry = 0.f;
  float4 cur = make_float4(0.f, 0.f, 0.f, 0.f);
  float cur_cost = kCostInf;
  int cur_sup = 0;
  if (inside) {
    rw = tile_window<H>(J, ref, x, y);
    fill_pcache(J, pc, x, y, &rx, &ry);
    cur = J.hyp[idx];
    cur_cost = J.cost[idx];
    cur_sup = J.support[idx];
  }
  const float ifx = 1.0f / J.rfx, ify = 1.0f / J.rfy;
  int counts[3] = {0, 0, 0};  // hypotheses, source windows sampled, of them read from a staged box
  float4 last = make_float4(-1.f, 0.f, 0.f, 0.f);
  Rng g{0};
  const float scale = exp2f(-(float)iter);
  const float span = J.rho_max - J.rho_min;
  // slots 0-7: propagation regions; 8-12: refinement candidates (one loop,
  // so that the hypothesis evaluation is instantiated once)
  for (int slot = 0; slot < 13; ++slot) {
    if (slot == 8) g = pixel_rng(J, idx, iter, 2 + color);
    float4 cand = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool have =
        inside && (slot < 8 ? propagation_candidate(J, x, y, slot, rx, ry, ifx, ify, cur, last, &cand)
                            : refinement_candidate(J, g, slot - 8, cur, rx, ry, scale, span, &cand) &&
                                  exploring(J, slot - 8, iter));
    const HypCost c = eval_plane_hyp_staged<H>(J, pc, x, y, rx, ry, cand, have, rw, ref, counts,
                                               J.prune ? cur_cost : kCostInf, wb);
    if (have && c.cost < cur_cost) {
      cur_cost = c.cost;
      cur = cand;
      cur_sup = c.support;
    }
  }
  if (J.eval_counter) add_counts(J, 0xffffffffu, counts, 3);
  if (inside) {
    J.hyp[idx] = cur;
    J.cost[idx] = cur_cost;
    J.support[idx] = (uint8_t)min(cur_sup, 255);
  }
}

// One red-black half-sweep over a whole batch: a persistent kernel (grid =
// resident blocks) whose blocks pull work items -- 64-column x R-row tiles,
// R = blockDim.y -- from an atomic counter until the batch is exhausted.  A
// block of 32 x R threads owns the 32 same-colour pixels of each of its R
// rows; the reference rows the tile reads (R + 2H rows, the 64 columns, 16
// more on the left and 32 on the right) are staged once into shared memory as
// even / odd column planes from the de-interleaved reference copy.
//
// A warp owns a compact patch, not a row: RW = min(R, 4) rows x 32 / RW
// same-colour pixels (16 x 4 pixels for R >= 4).  Each window sample of a
// warp is one texture instruction over its 32 pixels, and their source
// footprints then cluster in a 2-D patch of the source instead of spreading
// along a 64-pixel row: fewer texture-cache lines per instruction.  `queue`
// is this launch's work counter (zeroed by the init kernel); `total` its item
// count -- jobs with fewer iterations than `iter + 1` sit at the end of the
// job order and fall outside it.
//
// kStaged (exact interpolation, H > 0): the staged-window schedule -- each
// warp owns a kStageW x kStageH box of texel pairs at the start of the
// dynamic shared memory (the source-ray cache follows it) and reads the
// windows its pixels share from there (eval_view_staged).
template <int H, int kMode, bool kStaged>
__global__ void __maxnreg__(kStaged ? 128 : 96) k_plane_sweep(const __grid_constant__ PlaneBatch B, int total, int* queue, int color,
                                              int iter) {
  static_assert(!kStaged || (H > 0 && kMode == kSrcExact), "the staged schedule reads exact 2x2 footprints");
  extern __shared__ float2 smem[];
  constexpr int kHalo = H > 0 ? H : 1;
  __shared__ __align__(128) float tile[2 * (kMaxTileRows + 2 * kHalo) * kTileCols];
  __shared__ __align__(8) uint64_t bar;
  __shared__ __align__(8) uint64_t box_bar[kStaged ? kMaxTileRows : 1];
  __shared__ int s_item;
  const int R = (int)blockDim.y;
  const int nthreads = 32 * R;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  float2* pc_base = smem;
  WarpBox wb{nullptr, nullptr, 0u, 0, B.err, false};
  if constexpr (kStaged) {
    // the boxes first, from the first 128-byte boundary (TMA destinations)
    const uint32_t a = smem_addr(smem);
    char* boxes = reinterpret_cast<char*>(smem) + (((a + 127u) & ~127u) - a);
    wb.box = reinterpret_cast<float2*>(boxes + (size_t)threadIdx.y * kStageBytes);
    wb.bar = &box_bar[threadIdx.y];
    wb.polls = B.tma_poll_limit > 0 ? B.tma_poll_limit : kTmaWaitPolls;
    pc_base = reinterpret_cast<float2*>(boxes + (size_t)R * kStageBytes);
    if (threadIdx.x == 0) mbar_init(wb.bar, 1);
  }
  const PCache pc{pc_base, nthreads, tid};
  const int box_rows = R + 2 * H;
  // this thread's pixel in the tile: row ty, same-colour column pair `pair`.
  // A warp covers RW rows x PW pairs; within it each quad of lanes (the
  // texture unit's unit of work) takes 2 rows x 2 pairs -- a compact 4 x 2
  // pixel diamond whose source footprints share texture-cache sectors --
  // rather than 4 pairs of one row.
  const int RW = R < 4 ? R : 4;        // rows per warp
  const int PW = 32 / RW;              // pixels per warp row
  const int w = (int)threadIdx.y, l = (int)threadIdx.x;
  int r_in, c_in;
  if (RW == 4) {
    r_in = ((l >> 4) << 1) | ((l >> 1) & 1);
    c_in = (((l >> 2) & 3) << 1) | (l & 1);
  } else if (RW == 2) {
    r_in = (l >> 1) & 1;
    c_in = ((l >> 2) << 1) | (l & 1);
  } else {
    r_in = 0;
    c_in = l;
  }
  const int ty = (w / RW) * RW + r_in;
  const int pair = (w % RW) * PW + c_in;
  if constexpr (H > 0) {
    if (tid == 0) mbar_init(&bar, 1);
    __syncthreads();
  }
  uint32_t phase = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    const int j = find_job(B, item);
    const Job& J = B.jobs[j];
    const int local = item - B.start[j];
    const int tiles_x = (J.w + 63) >> 6;
    const int bx = local % tiles_x, by = local / tiles_x;
    const int y = by * R + ty;
    const int parity = (y + color) & 1;
    const int x = bx * 64 + 2 * pair + parity;
    if constexpr (H > 0) {
      // the tile: planes [2][box_rows][kTileCols] of ref_de from column bx*32 - 8 and
      // row by*R - H, one TMA box (zeros outside the image)
      const int polls = B.tma_poll_limit > 0 ? B.tma_poll_limit : kTmaWaitPolls;
      if (tid == 0 && !B.tma_skip)
        tma_load_3d(tile, B.tmaps + j, bx * 32 - 8, by * R - H, 0, &bar,
                    (uint32_t)(2 * box_rows * kTileCols * sizeof(float)));
      const bool ok = mbar_wait(&bar, phase, polls);
      phase ^= 1u;
      if (__syncthreads_or(!ok)) {
        // give the copy one more bounded chance to land before leaving
        if (tid == 0) {
          atomicExch(B.err, 1);
          mbar_wait(&bar, phase ^ 1u, polls);
        }
        break;
      }
    }
    const bool inside = x < J.w && y < J.h;
    if constexpr (kStaged) {
      const float* plane0 = tile;
      const float* plane1 = tile + box_rows * kTileCols;
      const TileRef ref{parity ? plane1 : plane0, parity ? plane0 : plane1, pair, parity, ty};
      sweep_pixel_staged<H>(J, pc, ref, inside, x, y, color, iter + J.iter_offset, wb);
    } else if (inside) {
      if constexpr (H > 0) {
        const float* plane0 = tile;
        const float* plane1 = tile + box_rows * kTileCols;
        const TileRef ref{parity ? plane1 : plane0, parity ? plane0 : plane1, pair, parity, ty};
        const RefWindow rw = tile_window<H>(J, ref, x, y);
        sweep_pixel<H, kMode>(J, pc, ref, rw, x, y, color, iter + J.iter_offset);
      } else {
        const GlobalRef ref{J.pref, J.w, x, y};
        const RefWindow rw = ref_window(J, x, y, J.half_pixel);
        sweep_pixel<H, kMode>(J, pc, ref, rw, x, y, color, iter + J.iter_offset);
      }
    }
    __syncthreads();
  }
  if constexpr (kStaged) {
    // a box copy whose wait ran out gets one more bounded chance to land
    // before the block's shared memory is released
    if (wb.dead && threadIdx.x == 0) mbar_wait(wb.bar, wb.phase ^ 1u, wb.polls);
  }
}

// Final maps of every job of the batch.
__global__ void __launch_bounds__(128) k_plane_output(const __grid_constant__ PlaneBatch B) {
  int j, x, y;
  if (!pixel_item(B, &j, &x, &y)) return;
  const Job& J = B.jobs[j];
  const int idx = y * J.w + x;
  const float4 h = J.hyp[idx];
  const float c = J.cost[idx];
  float d = __int_as_float(0x7fc00000);
  float cf = 0.f;
  uint8_t sp = 0;
  if (c < 1e29f && h.x > 0.f) {
    const float dd = 1.0f / h.x;
    if (dd >= (float)J.min_depth && dd <= (float)J.max_depth) {
      d = dd;
      cf = 1.0f - fminf(1.0f, fmaxf(0.0f, c));
      sp = J.support[idx];
      atomicAdd(J.out_filled, 1u);
    }
  }
  J.out_depth[idx] = d;
  J.out_support[idx] = sp;
  J.out_conf[idx] = cf;
  if (J.out_normal) {
    J.out_normal[3 * idx] = h.y;
    J.out_normal[3 * idx + 1] = h.z;
    J.out_normal[3 * idx + 2] = h.w;
  }
  if (J.out_cost) J.out_cost[idx] = c;
}

// ---------------------------------------------------------------------------
// compat mode (the reference algorithm)
// ---------------------------------------------------------------------------
__global__ void k_compat_init(Job J, float* cost) {
  extern __shared__ float2 smem[];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  PCache pc{smem, (int)(blockDim.x * blockDim.y), tid};
  if (x >= J.w || y >= J.h) return;
  const int idx = y * J.w + x;
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  const RefWindow rw = ref_window(J, x, y, true);
  const HypCost c = eval_compat_hyp(J, pc, x, y, J.inv[idx], rw, nullptr);
  cost[idx] = c.cost;
  J.isupport[idx] = c.support;
}

// One direction sweep (patchmatch_stereo.cpp:642-723) for every pixel at
// once: candidates come from the snapshot (inv_in, cost_in); the pixel's own
// draws -- random_search_count signed draws, the restart flag and the
// restart draw -- were generated on the host in the reference's scan order.
__global__ void k_compat_sweep(Job J, const double* __restrict__ inv_in, const float* __restrict__ cost_in,
                               const int32_t* __restrict__ sup_in, double* inv_out, float* cost_out,
                               int32_t* sup_out, const uint32_t* __restrict__ draws, const uint8_t* __restrict__ fire,
                               int draw_stride, int search_count, double radius_ratio, int propagate) {
  extern __shared__ float2 smem[];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  PCache pc{smem, (int)(blockDim.x * blockDim.y), tid};
  if (x >= J.w || y >= J.h) return;
  const int idx = y * J.w + x;
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  const RefWindow rw = ref_window(J, x, y, true);
  double out_inv = inv_in[idx];
  float out_cost = cost_in[idx];
  int out_sup = sup_in[idx];
  if (propagate) {
    const int nbx[4] = {-1, 1, 0, 0}, nby[4] = {0, 0, -1, 1};
    for (int k = 0; k < 4; ++k) {
      const int nx_ = x + nbx[k], ny_ = y + nby[k];
      if (nx_ < 0 || ny_ < 0 || nx_ >= J.w || ny_ >= J.h) continue;
      const int n = ny_ * J.w + nx_;
      if (cost_in[n] >= 1e29f) continue;
      const double cand = inv_in[n];
      const HypCost c = eval_compat_hyp(J, pc, x, y, cand, rw, nullptr);
      if (c.cost < out_cost) {
        out_cost = c.cost;
        out_inv = cand;
        out_sup = c.support;
      }
    }
  }
  const uint32_t* d = draws + (size_t)idx * draw_stride;
  double radius = out_inv * radius_ratio;
  for (int k = 0; k < search_count; ++k) {
    const double sgn = ((double)d[k] / 4294967296.0) * 2.0 - 1.0;
    const double cand = out_inv + sgn * radius;
    if (cand < J.dinv_min || cand > J.dinv_max) {
      radius *= 0.5;
      continue;
    }
    const HypCost c = eval_compat_hyp(J, pc, x, y, cand, rw, nullptr);
    if (c.cost < out_cost) {
      out_cost = c.cost;
      out_inv = cand;
      out_sup = c.support;
    }
    radius *= 0.5;
  }
  if (fire[idx]) {
    const double cand = J.dinv_min + ((double)d[search_count] / 4294967296.0) * (J.dinv_max - J.dinv_min);
    const HypCost c = eval_compat_hyp(J, pc, x, y, cand, rw, nullptr);
    if (c.cost < out_cost) {
      out_cost = c.cost;
      out_inv = cand;
      out_sup = c.support;
    }
  }
  inv_out[idx] = out_inv;
  cost_out[idx] = out_cost;
  sup_out[idx] = out_sup;
}

// patchmatch_stereo.cpp:744-763
__global__ void k_compat_output(Job J, const double* __restrict__ inv, const float* __restrict__ cost,
                                const int32_t* __restrict__ sup, float* depth, uint8_t* support, float* conf,
                                unsigned int* filled) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= J.w || y >= J.h) return;
  const int idx = y * J.w + x;
  float d = __int_as_float(0x7fc00000);
  float cf = 0.f;
  uint8_t sp = 0;
  if (cost[idx] < 1e29f) {
    const double iv = inv[idx];
    const double dd = iv <= 1e-9 ? 1e9 : 1.0 / iv;
    if (!(dd < J.min_depth || dd > J.max_depth)) {
      d = (float)dd;
      sp = (uint8_t)min(sup[idx], 255);
      const double pc = fmin(1.0, fmax(0.0, (double)cost[idx]));
      cf = (float)(1.0 - pc);
      atomicAdd(filled, 1u);
    }
  }
  depth[idx] = d;
  support[idx] = sp;
  conf[idx] = cf;
}

// RefineSubpixel (patchmatch_stereo.cpp:770-979), one thread per pixel.
// Inverse-depth arithmetic in FP64 as in the reference; costs FP32.
__device__ __forceinline__ bool solve3(const double A[3][3], const double b[3], double x[3]) {
  double m[3][4];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) m[i][j] = A[i][j];
    m[i][3] = b[i];
  }
  for (int col = 0; col < 3; ++col) {
    int pivot = col;
    for (int r = col + 1; r < 3; ++r)
      if (fabs(m[r][col]) > fabs(m[pivot][col])) pivot = r;
    if (fabs(m[pivot][col]) < 1e-18) return false;
    if (pivot != col)
      for (int j = 0; j < 4; ++j) {
        const double t = m[col][j];
        m[col][j] = m[pivot][j];
        m[pivot][j] = t;
      }
    for (int r = 0; r < 3; ++r) {
      if (r == col) continue;
      const double f = m[r][col] / m[col][col];
      for (int j = col; j < 4; ++j) m[r][j] -= f * m[col][j];
    }
  }
  for (int i = 0; i < 3; ++i) {
    if (fabs(m[i][i]) < 1e-18) return false;
    x[i] = m[i][3] / m[i][i];
  }
  return true;
}

__global__ void k_compat_refine(Job J, float* depth, float* conf, double inv_per_px, int fit_points_cfg,
                                int subpixel_iterations, unsigned int* refined, double* out_best_inv,
                                float* out_best_cost) {
  extern __shared__ float2 smem[];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  PCache pc{smem, (int)(blockDim.x * blockDim.y), tid};
  if (x >= J.w || y >= J.h) return;
  const int idx = y * J.w + x;
  const float d0 = depth[idx];
  if (out_best_inv) {
    out_best_inv[idx] = __longlong_as_double(0x7ff8000000000000ll);
    out_best_cost[idx] = kCostInf;
  }
  if (!isfinite(d0)) return;
  const double inv0 = (double)d0 < 1e-9 ? 1e9 : 1.0 / (double)d0;
  if (inv0 < J.dinv_min || inv0 > J.dinv_max) return;
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  const RefWindow rw = ref_window(J, x, y, true);
  auto eval = [&](double v) -> float { return eval_compat_hyp(J, pc, x, y, v, rw, nullptr).cost; };
  const int fit_points = fit_points_cfg > 3 ? fit_points_cfg : 3;
  const int half_fit = fit_points / 2;
  const double fit_step = inv_per_px * 0.5;
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, t0 = 0, t1 = 0, t2 = 0;
  bool fit_ok = fit_points <= 64;
  for (int k = 0; k < fit_points && fit_ok; ++k) {
    const double dk = inv0 + (k - half_fit) * fit_step;
    if (dk < J.dinv_min || dk > J.dinv_max) {
      fit_ok = false;
      break;
    }
    const double c = (double)eval(dk);
    if (c >= 1e29) fit_ok = false;
    const double xx = (double)(k - half_fit);
    s0 += 1.0;
    s1 += xx;
    s2 += xx * xx;
    s3 += xx * xx * xx;
    s4 += xx * xx * xx * xx;
    t0 += c;
    t1 += xx * c;
    t2 += xx * xx * c;
  }
  double best_d = inv0;
  float best_c = eval(inv0);
  if (fit_ok) {
    const double A[3][3] = {{s4, s3, s2}, {s3, s2, s1}, {s2, s1, s0}};
    const double b[3] = {t2, t1, t0};
    double sol[3];
    if (solve3(A, b, sol) && fabs(sol[0]) > 1e-12) {
      const double vertex = -sol[1] / (2.0 * sol[0]);
      // the vertex is in sample-index units and is added unscaled, as in
      // the reference (patchmatch_stereo.cpp:896-899)
      if (vertex >= -(double)half_fit && vertex <= (double)half_fit) {
        const double cand = inv0 + vertex;
        const float cc = eval(cand);
        if (cc < best_c) {
          best_c = cc;
          best_d = cand;
        }
      }
    }
  }
  {
    double lo = best_d - inv_per_px * 1.0;
    double hi = best_d + inv_per_px * 1.0;
    if (lo < J.dinv_min) lo = J.dinv_min;
    if (hi > J.dinv_max) hi = J.dinv_max;
    if (hi > lo) {
      const double inv_phi = 0.6180339887498949;
      double c1 = hi - inv_phi * (hi - lo);
      double c2 = lo + inv_phi * (hi - lo);
      float f1 = eval(c1), f2 = eval(c2);
      for (int k = 0; k < subpixel_iterations; ++k) {
        if (f1 < f2) {
          hi = c2;
          c2 = c1;
          f2 = f1;
          c1 = hi - inv_phi * (hi - lo);
          f1 = eval(c1);
        } else {
          lo = c1;
          c1 = c2;
          f1 = f2;
          c2 = lo + inv_phi * (hi - lo);
          f2 = eval(c2);
        }
      }
      const double mid = 0.5 * (lo + hi);
      const float cm = eval(mid);
      if (cm < best_c) {
        best_c = cm;
        best_d = mid;
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
  if (out_best_inv) {
    out_best_inv[idx] = best_d;
    out_best_cost[idx] = best_c;
  }
  if (best_d < J.dinv_min || best_d > J.dinv_max) return;
  const double fd = best_d <= 1e-9 ? 1e9 : 1.0 / best_d;
  if (fd < J.min_depth || fd > J.max_depth) return;
  depth[idx] = (float)fd;
  const double pcost = fmin(1.0, fmax(0.0, (double)best_c));
  conf[idx] = (float)(1.0 - pcost);
  atomicAdd(refined, 1u);
}

// Plane-mode refinement: golden-section search on the inverse depth along
// the pixel's own plane normal over +-1 px of disparity, the reference's
// refinement schedule applied to the plane cost.
template <int H, int kMode>
__global__ void __launch_bounds__(128, 4) k_plane_refine(const __grid_constant__ PlaneBatch B) {
  extern __shared__ float2 smem[];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  int j, x, y;
  if (!pixel_item(B, &j, &x, &y)) return;
  const Job& J = B.jobs[j];
  if (J.refine_iters <= 0 || J.refine_mode != 1) return;
  PCache pc{smem, 128, tid};
  const int idx = y * J.w + x;
  const float4 h0 = J.hyp[idx];
  const float c0 = J.cost[idx];
  if (!(c0 < 1e29f)) return;
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  const RefWindow rw = ref_window(J, x, y, J.half_pixel);
  const GlobalRef ref{J.pref, J.w, x, y};
  auto eval = [&](float v) -> HypCost {
    return eval_plane_hyp<H, kMode>(J, pc, x, y, rx, ry, v, h0.y, h0.z, h0.w, rw, ref, nullptr);
  };
  float best_d = h0.x, best_c = c0;
  int best_s = J.support[idx];
  float lo = fmaxf(J.rho_min, best_d - J.inv_per_px);
  float hi = fminf(J.rho_max, best_d + J.inv_per_px);
  if (hi > lo) {
    const float inv_phi = 0.618033988749895f;
    float c1 = hi - inv_phi * (hi - lo), c2 = lo + inv_phi * (hi - lo);
    HypCost f1 = eval(c1), f2 = eval(c2);
    for (int k = 0; k < J.refine_iters; ++k) {
      if (f1.cost < f2.cost) {
        hi = c2;
        c2 = c1;
        f2 = f1;
        c1 = hi - inv_phi * (hi - lo);
        f1 = eval(c1);
      } else {
        lo = c1;
        c1 = c2;
        f1 = f2;
        c2 = lo + inv_phi * (hi - lo);
        f2 = eval(c2);
      }
    }
    const float mid = 0.5f * (lo + hi);
    const HypCost fm = eval(mid);
    if (fm.cost < best_c) {
      best_c = fm.cost;
      best_d = mid;
      best_s = fm.support;
    }
    if (f1.cost < best_c) {
      best_c = f1.cost;
      best_d = c1;
      best_s = f1.support;
    }
    if (f2.cost < best_c) {
      best_c = f2.cost;
      best_d = c2;
      best_s = f2.support;
    }
  }
  J.hyp[idx] = make_float4(best_d, h0.y, h0.z, h0.w);
  J.cost[idx] = best_c;
  J.support[idx] = (uint8_t)min(best_s, 255);
}

// Plane-mode Gauss-Newton refinement (refine mode 2): Levenberg-Marquardt
// steps on (d, theta, phi) from the adjoint of the aggregated cost (exact
// bilinear reads, window recomputed per pass), each step accepted only when
// the search's own cost of the new plane is lower.
// The gradient and Gauss-Newton matrix of the aggregated cost for one
// refinement step: each view's moments (and from them the best_k selection)
// by the search's own window code with exact 2x2 reads -- an incremental
// homography walk -- then the adjoint's Jacobian pass over the selected
// views only.  False for an invalid hypothesis.
template <int H, int kMode, class Ref>
__device__ bool gn_gradient(const Job& J, const PCache& pc, int x, int y, float rx, float ry, const AdjHyp& h,
                            const RefWindow& rw, const Ref& ref, float g[3], float Hm[6]) {
  constexpr int kExact = kMode == kSrcBf16 ? kSrcBf16 : kSrcExact;
  for (int i = 0; i < 3; ++i) g[i] = 0.f;
  for (int i = 0; i < 6; ++i) Hm[i] = 0.f;
  PlaneHyp hp;
  if (!make_plane_hyp(J, rx, ry, 1.0f / h.d, h.n[0], h.n[1], h.n[2], &hp)) return false;
  const int ns = min(J.num_src, kMaxSources);
  ViewMom mom[kMaxSources];
  float vc[kMaxSources];
  int nvalid = 0;
  for (int s = 0; s < ns; ++s) {
    ff P[3];
    pc.get(s, P);
    float m[6];
    const ViewResult v = eval_view_plane<H, kExact>(J, J.src[s], x, y, P, hp, rw, ref, m);
    mom[s].valid = v.valid > 0;
    vc[s] = kCostInf;
    if (mom[s].valid) {
      mom[s].n = m[0];
      mom[s].mr = m[1];
      mom[s].ms = m[2];
      mom[s].srr = m[3];
      mom[s].sss = m[4];
      mom[s].srs = m[5];
      mom[s].ncc = v.ncc;
      vc[s] = 1.0f - v.ncc;
      ++nvalid;
    }
  }
  if (nvalid == 0) return false;
  const int k = (J.best_k <= 0 || J.best_k >= nvalid || J.best_k > kMaxBestK) ? nvalid : J.best_k;
  // the k lowest costs, ties to the lower source index
  uint32_t sel = 0;
  for (int t = 0; t < k; ++t) {
    int b = -1;
    for (int s = 0; s < ns; ++s)
      if (mom[s].valid && !((sel >> s) & 1u) && (b < 0 || vc[s] < vc[b])) b = s;
    sel |= 1u << b;
  }
  const float inv_k = 1.0f / (float)k;
  for (int s = 0; s < ns; ++s) {
    if (!((sel >> s) & 1u)) continue;
    float gs[3], Hs[6];
    const ViewGeo geo = view_geo(J, J.src[s], h);
    view_adjoint<kMode, false>(J, J.src[s], geo, h, mom[s], gs, Hs, nullptr, nullptr);
    for (int i = 0; i < 3; ++i) g[i] += gs[i] * inv_k;
    for (int i = 0; i < 6; ++i) Hm[i] += Hs[i] * inv_k;
  }
  return true;
}

template <int H, int kMode>
__global__ void __launch_bounds__(128, 5) k_plane_refine_gn(const __grid_constant__ PlaneBatch B) {
  extern __shared__ float2 smem[];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  int j, x, y;
  if (!pixel_item(B, &j, &x, &y)) return;
  const Job& J = B.jobs[j];
  if (J.refine_iters <= 0 || J.refine_mode != 2) return;
  PCache pc{smem, 128, tid};
  const int idx = y * J.w + x;
  const float4 h0 = J.hyp[idx];
  float cur = J.cost[idx];
  if (!(cur < 1e29f) || !(h0.x > 0.f)) return;
  int sup = J.support[idx];
  float rx, ry;
  fill_pcache(J, pc, x, y, &rx, &ry);
  const RefWindow rw = ref_window(J, x, y, J.half_pixel);
  const GlobalRef ref{J.pref, J.w, x, y};
  float d = 1.0f / h0.x;
  float theta = acosf(fminf(1.0f, fmaxf(-1.0f, h0.w))), phi = atan2f(h0.z, h0.y);
  float4 best = h0;
  float lambda = 1e-3f;
  for (int it = 0; it < J.refine_iters; ++it) {
    AdjHyp ah;
    if (!make_adj_hyp(J, x, y, d, theta, phi, &ah)) break;
    float g[3], Hm[6];
    if (!gn_gradient<H, kMode>(J, pc, x, y, rx, ry, ah, rw, ref, g, Hm)) break;
    bool accepted = false;
    for (int t = 0; t < 4 && !accepted; ++t) {
      float step[3];
      if (!solve_lm3(Hm, g, lambda, step)) {
        lambda *= 10.0f;
        continue;
      }
      const float nd = d + step[0], nt = theta + step[1], np = phi + step[2];
      float n[3], dt[3], dp[3];
      sph_normal(nt, np, n, dt, dp);
      const HypCost hc =
          eval_plane_hyp<H, kMode>(J, pc, x, y, rx, ry, 1.0f / nd, n[0], n[1], n[2], rw, ref, nullptr, nullptr,
                                   J.prune ? cur : kCostInf);
      if (nd > 0.f && hc.cost < cur) {
        d = nd;
        theta = nt;
        phi = np;
        cur = hc.cost;
        sup = hc.support;
        best = make_float4(1.0f / nd, n[0], n[1], n[2]);
        lambda *= 0.3f;
        accepted = true;
      } else {
        lambda *= 10.0f;
      }
    }
    if (!accepted) break;
  }
  J.hyp[idx] = best;
  J.cost[idx] = cur;
  J.support[idx] = (uint8_t)min(sup, 255);
}

// ---------------------------------------------------------------------------
// image preparation
// ---------------------------------------------------------------------------
__global__ void k_prep_ref(const uint8_t* __restrict__ img, int w, int h, float* ref, float* box) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const float v = (float)img[y * w + x] - 128.0f;
  ref[y * w + x] = v;
  if (box) {
    // the reference's window sample at (x + 0.5, y + 0.5): an exact 2x2
    // average; defined for x <= w-2, y <= h-2 (SampleBilinear's range)
    const int x1 = min(x + 1, w - 1), y1 = min(y + 1, h - 1);
    const float s = (float)img[y * w + x] + (float)img[y * w + x1] + (float)img[y1 * w + x] + (float)img[y1 * w + x1];
    box[y * w + x] = 0.25f * s - 128.0f;
  }
}

// Even / odd column planes of the (I - 128) reference image:
// out[p][y][i] = ref[y][2i + p] for i < half_w (0 past the right edge), rows
// of `pitch` floats (the padding is zero).
__global__ void k_deinterleave(const float* __restrict__ ref, int w, int h, int half_w, int pitch, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= pitch || y >= h) return;
  for (int p = 0; p < 2; ++p) {
    const int x = 2 * i + p;
    out[((size_t)p * h + y) * pitch + i] = (i < half_w && x < w) ? ref[(size_t)y * w + x] : 0.f;
  }
}

// One staged source texel of (I - 128) in the storage format (0 FP32, 1 FP16,
// 2 BF16 bits), rounded to nearest even.
// One source texel, v = I - 128, in the storage format (0 FP32, 1 FP16,
// 2 BF16 bits, 3 the 8-bit intensity I rounded to nearest and clamped).
__device__ __forceinline__ void store_texel(void* out, size_t i, float v, int storage) {
  if (storage == 1)
    ((__half*)out)[i] = __float2half_rn(v);
  else if (storage == 2)
    ((unsigned short*)out)[i] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
  else if (storage == 3)
    ((uint8_t*)out)[i] = (uint8_t)__float2int_rn(fminf(255.0f, fmaxf(0.0f, v + 128.0f)));
  else
    ((float*)out)[i] = v;
}

__global__ void k_prep_src(const uint8_t* __restrict__ img, int w, int h, void* out, size_t pitch_elems,
                           int storage) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  store_texel(out, y * pitch_elems + x, (float)img[y * w + x] - 128.0f, storage);
}

__global__ void k_prep_ref_f32(const float* __restrict__ img, int w, int h, float* ref, float* box) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  ref[y * w + x] = img[y * w + x] - 128.0f;
  if (box) {
    const int x1 = min(x + 1, w - 1), y1 = min(y + 1, h - 1);
    const float s = (img[y * w + x] + img[y * w + x1]) + (img[y1 * w + x] + img[y1 * w + x1]);
    box[y * w + x] = 0.25f * s - 128.0f;
  }
}

__global__ void k_prep_src_f32in(const float* __restrict__ img, int w, int h, void* out, size_t pitch_elems,
                                 int storage) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  store_texel(out, y * pitch_elems + x, img[y * w + x] - 128.0f, storage);
}

// ComputeNcc (patchmatch_stereo.cpp:214-274) for a batch of windows, FP64 in
// the reference's operation order: a standalone API, not the hot path.
__device__ __forceinline__ bool sample_bilinear_d(const uint8_t* img, int w, int h, double u, double v, double* out) {
  if (u < 0.0 || v < 0.0 || u > (double)(w - 1) || v > (double)(h - 1)) return false;
  const int x0 = (int)floor(u), y0 = (int)floor(v);
  const int x1 = min(x0 + 1, w - 1), y1 = min(y0 + 1, h - 1);
  const double fx = __dsub_rn(u, (double)x0), fy = __dsub_rn(v, (double)y0);
  const double p00 = img[y0 * w + x0], p10 = img[y0 * w + x1], p01 = img[y1 * w + x0], p11 = img[y1 * w + x1];
  const double top = __dadd_rn(__dmul_rn(p00, __dsub_rn(1.0, fx)), __dmul_rn(p10, fx));
  const double bot = __dadd_rn(__dmul_rn(p01, __dsub_rn(1.0, fx)), __dmul_rn(p11, fx));
  *out = __dadd_rn(__dmul_rn(top, __dsub_rn(1.0, fy)), __dmul_rn(bot, fy));
  return true;
}

__global__ void k_ncc_windows(const uint8_t* __restrict__ ref, int ref_w, int ref_h, const uint8_t* __restrict__ src,
                              int src_w, int src_h, int patch_size, int n, const NccWindow* __restrict__ win,
                              int* valid_out, double* ncc_out, int* weak_out, int* samples_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const NccWindow w = win[i];
  const int half = patch_size / 2;
  double sr = 0, ss = 0, srr = 0, sss = 0, srs = 0;
  int valid = 0;
  for (int dy = -half; dy <= half; ++dy)
    for (int dx = -half; dx <= half; ++dx) {
      double vr, vs;
      if (!sample_bilinear_d(ref, ref_w, ref_h, __dadd_rn(w.ref_u, (double)dx), __dadd_rn(w.ref_v, (double)dy), &vr))
        continue;
      if (!sample_bilinear_d(src, src_w, src_h, __dadd_rn(w.src_u, (double)dx), __dadd_rn(w.src_v, (double)dy), &vs))
        continue;
      sr = __dadd_rn(sr, vr);
      ss = __dadd_rn(ss, vs);
      srr = __dadd_rn(srr, __dmul_rn(vr, vr));
      sss = __dadd_rn(sss, __dmul_rn(vs, vs));
      srs = __dadd_rn(srs, __dmul_rn(vr, vs));
      ++valid;
    }
  int ok = 0, weak = 0;
  double ncc = 0.0;
  if (valid >= patch_size * patch_size / 2) {
    const double nn = (double)valid;
    const double mr = __ddiv_rn(sr, nn), ms = __ddiv_rn(ss, nn);
    const double var_r = __dsub_rn(__ddiv_rn(srr, nn), __dmul_rn(mr, mr));
    const double var_s = __dsub_rn(__ddiv_rn(sss, nn), __dmul_rn(ms, ms));
    weak = var_r < 12.0;
    const double denom = __dsqrt_rn(__dmul_rn(var_r, var_s));
    if (!(denom < 1e-9)) {
      ncc = __ddiv_rn(__dsub_rn(__ddiv_rn(srs, nn), __dmul_rn(mr, ms)), denom);
      ncc = fmin(1.0, fmax(-1.0, ncc));
      ok = 1;
    }
  }
  valid_out[i] = ok;
  ncc_out[i] = ok ? ncc : 0.0;
  weak_out[i] = weak;
  samples_out[i] = ok ? valid : 0;
}


// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static size_t pcache_bytes(int num_src, int threads) { return (size_t)num_src * 3 * threads * sizeof(float2); }

static dim3 grid2d(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

// Dynamic shared memory above the 48 KB default needs an opt-in per kernel.
template <class K>
static cudaError_t allow_smem(K* kernel, size_t bytes) {
  if (bytes <= 32 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Calls f(integral_constant<H>, integral_constant<kMode>) for the compiled
// window sizes (11x11, 7x7, and the generic runtime-size path) and source
// modes; BF16 sources have the 11x11 and generic instances only.
template <class F>
static cudaError_t dispatch_plane(int patch_half, int mode, F&& f) {
  using std::integral_constant;
  if (mode == kSrcTex) {
    if (patch_half == 5) return f(integral_constant<int, 5>{}, integral_constant<int, kSrcTex>{});
    if (patch_half == 3) return f(integral_constant<int, 3>{}, integral_constant<int, kSrcTex>{});
    return f(integral_constant<int, 0>{}, integral_constant<int, kSrcTex>{});
  }
  if (mode == kSrcBf16) {
    if (patch_half == 5) return f(integral_constant<int, 5>{}, integral_constant<int, kSrcBf16>{});
    return f(integral_constant<int, 0>{}, integral_constant<int, kSrcBf16>{});
  }
  if (patch_half == 5) return f(integral_constant<int, 5>{}, integral_constant<int, kSrcExact>{});
  if (patch_half == 3) return f(integral_constant<int, 3>{}, integral_constant<int, kSrcExact>{});
  return f(integral_constant<int, 0>{}, integral_constant<int, kSrcExact>{});
}

cudaError_t launch_eval_hyps(const Job& J, int mode, int n, const int* px, const int* py, const double* inv,
                             const float* normals, float* cost, int* support, float* view_cost, cudaStream_t st) {
  const int threads = 128;
  const int blocks = (n + threads - 1) / threads;
  if (blocks == 0) return cudaSuccess;
  const size_t sm = pcache_bytes(J.num_src, threads);
  return dispatch_plane(J.patch_half, J.src_mode, [&](auto h, auto k) {
    auto* fn = k_eval_hyps<decltype(h)::value, decltype(k)::value>;
    cudaError_t e = allow_smem(fn, sm);
    if (e != cudaSuccess) return e;
    fn<<<blocks, threads, sm, st>>>(J, mode, n, px, py, inv, normals, cost, support, view_cost);
    return cudaGetLastError();
  });
}

cudaError_t launch_plane_init(const PlaneBatch& B, int patch_half, int mode, int max_src, int* queues, int num_queues,
                              cudaStream_t st) {
  const int total = B.start[B.njobs];
  if (total <= 0) return cudaSuccess;
  const size_t sm = pcache_bytes(max_src, 128);
  return dispatch_plane(patch_half, mode, [&](auto h, auto k) {
    auto* fn = k_plane_init<decltype(h)::value, decltype(k)::value>;
    cudaError_t e = allow_smem(fn, sm);
    if (e != cudaSuccess) return e;
    fn<<<total, dim3(32, 4), sm, st>>>(B, queues, num_queues);
    return cudaGetLastError();
  });
}

// The staged schedule's dynamic shared memory: the warps' boxes (after up to
// 128 bytes of alignment) and then the source-ray cache.
static size_t sweep_smem_bytes(int max_src, int rows, bool staged) {
  return pcache_bytes(max_src, 32 * rows) + (staged ? 128 + (size_t)rows * kStageBytes : 0);
}

// Calls f(kernel) for the sweep instance of (window, mode, schedule).
template <class F>
static cudaError_t dispatch_sweep(int patch_half, int mode, int staged, F&& f) {
  if (staged) {
    if (mode != kSrcExact) return cudaErrorInvalidValue;
    if (patch_half == 5) return f(k_plane_sweep<5, kSrcExact, true>);
    if (patch_half == 3) return f(k_plane_sweep<3, kSrcExact, true>);
    return cudaErrorInvalidValue;
  }
  return dispatch_plane(patch_half, mode, [&](auto h, auto k) {
    return f(k_plane_sweep<decltype(h)::value, decltype(k)::value, false>);
  });
}

cudaError_t plane_sweep_occupancy(int patch_half, int mode, int max_src, int rows, int staged, int* blocks_per_sm) {
  const size_t sm = sweep_smem_bytes(max_src, rows, staged != 0);
  return dispatch_sweep(patch_half, mode, staged, [&](auto* fn) {
    cudaError_t e = allow_smem(fn, sm);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, 32 * rows, sm);
  });
}

cudaError_t launch_plane_sweep(const PlaneBatch& B, int total, int* queue, int patch_half, int mode, int max_src,
                               int rows, int staged, int grid, int color, int iter, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  if (rows < 1 || rows > kMaxTileRows || grid < 1 || total > B.start[B.njobs]) return cudaErrorInvalidValue;
  const size_t sm = sweep_smem_bytes(max_src, rows, staged != 0);
  return dispatch_sweep(patch_half, mode, staged, [&](auto* fn) {
    cudaError_t e = allow_smem(fn, sm);
    if (e != cudaSuccess) return e;
    fn<<<grid, dim3(32, rows), sm, st>>>(B, total, queue, color, iter);
    return cudaGetLastError();
  });
}

__global__ void k_pair_image(cudaTextureObject_t tex, int w, int h, float2* out, int pitch) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const float a = tex2D<float>(tex, (float)x + 0.5f, (float)y + 0.5f);
  const float b = x + 1 < w ? tex2D<float>(tex, (float)x + 1.5f, (float)y + 0.5f) : 0.0f;
  out[(size_t)y * pitch + x] = make_float2(a, b);
}

cudaError_t launch_pair_image(cudaTextureObject_t tex, int w, int h, float2* out, int pitch, cudaStream_t st) {
  if (w < 1 || h < 1 || pitch < w) return cudaErrorInvalidValue;
  const dim3 b(32, 8);
  k_pair_image<<<grid2d(w, h, b), b, 0, st>>>(tex, w, h, out, pitch);
  return cudaGetLastError();
}

cudaError_t launch_plane_refine(const PlaneBatch& B, int patch_half, int mode, int max_src, cudaStream_t st) {
  const int total = B.start[B.njobs];
  if (total <= 0) return cudaSuccess;
  const size_t sm = pcache_bytes(max_src, 128);
  return dispatch_plane(patch_half, mode, [&](auto h, auto k) {
    auto* fn = k_plane_refine<decltype(h)::value, decltype(k)::value>;
    cudaError_t e = allow_smem(fn, sm);
    if (e != cudaSuccess) return e;
    fn<<<total, dim3(32, 4), sm, st>>>(B);
    return cudaGetLastError();
  });
}

cudaError_t launch_plane_refine_gn(const PlaneBatch& B, int patch_half, int mode, int max_src, cudaStream_t st) {
  const int total = B.start[B.njobs];
  if (total <= 0) return cudaSuccess;
  const size_t sm = pcache_bytes(max_src, 128);
  return dispatch_plane(patch_half, mode, [&](auto h, auto k) {
    auto* fn = k_plane_refine_gn<decltype(h)::value, decltype(k)::value>;
    cudaError_t e = allow_smem(fn, sm);
    if (e != cudaSuccess) return e;
    fn<<<total, dim3(32, 4), sm, st>>>(B);
    return cudaGetLastError();
  });
}

cudaError_t launch_plane_output(const PlaneBatch& B, cudaStream_t st) {
  const int total = B.start[B.njobs];
  if (total <= 0) return cudaSuccess;
  k_plane_output<<<total, dim3(32, 4), 0, st>>>(B);
  return cudaGetLastError();
}

cudaError_t launch_compat_init(const Job& J, float* cost, cudaStream_t st) {
  const dim3 b(32, 4);
  k_compat_init<<<grid2d(J.w, J.h, b), b, pcache_bytes(J.num_src, 128), st>>>(J, cost);
  return cudaGetLastError();
}

cudaError_t launch_compat_sweep(const Job& J, const double* inv_in, const float* cost_in, const int32_t* sup_in,
                                double* inv_out, float* cost_out, int32_t* sup_out, const uint32_t* draws,
                                const uint8_t* fire, int draw_stride, int search_count, double radius_ratio,
                                int propagate, cudaStream_t st) {
  const dim3 b(32, 4);
  k_compat_sweep<<<grid2d(J.w, J.h, b), b, pcache_bytes(J.num_src, 128), st>>>(
      J, inv_in, cost_in, sup_in, inv_out, cost_out, sup_out, draws, fire, draw_stride, search_count, radius_ratio,
      propagate);
  return cudaGetLastError();
}

cudaError_t launch_compat_output(const Job& J, const double* inv, const float* cost, const int32_t* sup, float* depth,
                                 uint8_t* support, float* conf, unsigned int* filled, cudaStream_t st) {
  const dim3 b(32, 8);
  k_compat_output<<<grid2d(J.w, J.h, b), b, 0, st>>>(J, inv, cost, sup, depth, support, conf, filled);
  return cudaGetLastError();
}

cudaError_t launch_compat_refine(const Job& J, float* depth, float* conf, double inv_per_px, int fit_points,
                                 int iters, unsigned int* refined, double* best_inv, float* best_cost,
                                 cudaStream_t st) {
  const dim3 b(32, 4);
  k_compat_refine<<<grid2d(J.w, J.h, b), b, pcache_bytes(J.num_src, 128), st>>>(
      J, depth, conf, inv_per_px, fit_points, iters, refined, best_inv, best_cost);
  return cudaGetLastError();
}

cudaError_t launch_prep_ref(const uint8_t* img, int w, int h, float* ref, float* box, cudaStream_t st) {
  const dim3 b(32, 8);
  k_prep_ref<<<grid2d(w, h, b), b, 0, st>>>(img, w, h, ref, box);
  return cudaGetLastError();
}

static size_t texel_bytes(int storage) { return storage == 0 ? 4 : storage == 3 ? 1 : 2; }

cudaError_t launch_prep_src(const uint8_t* img, int w, int h, void* out, size_t pitch_bytes, int storage,
                            cudaStream_t st) {
  const dim3 b(32, 8);
  k_prep_src<<<grid2d(w, h, b), b, 0, st>>>(img, w, h, out, pitch_bytes / texel_bytes(storage), storage);
  return cudaGetLastError();
}

cudaError_t launch_prep_ref_f32(const float* img, int w, int h, float* ref, float* box, cudaStream_t st) {
  const dim3 b(32, 8);
  k_prep_ref_f32<<<grid2d(w, h, b), b, 0, st>>>(img, w, h, ref, box);
  return cudaGetLastError();
}

cudaError_t launch_prep_src_f32in(const float* img, int w, int h, void* out, size_t pitch_bytes, int storage,
                                  cudaStream_t st) {
  const dim3 b(32, 8);
  k_prep_src_f32in<<<grid2d(w, h, b), b, 0, st>>>(img, w, h, out, pitch_bytes / texel_bytes(storage), storage);
  return cudaGetLastError();
}

cudaError_t launch_ncc_windows(const uint8_t* ref, int ref_w, int ref_h, const uint8_t* src, int src_w, int src_h,
                               int patch_size, int n, const NccWindow* win, int* valid, double* ncc, int* weak,
                               int* samples, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_ncc_windows<<<(n + 127) / 128, 128, 0, st>>>(ref, ref_w, ref_h, src, src_w, src_h, patch_size, n, win, valid, ncc,
                                                 weak, samples);
  return cudaGetLastError();
}

cudaError_t launch_deinterleave(const float* ref, int w, int h, int half_w, int pitch, float* out, cudaStream_t st) {
  const dim3 b(32, 8);
  k_deinterleave<<<grid2d(pitch, h, b), b, 0, st>>>(ref, w, h, half_w, pitch, out);
  return cudaGetLastError();
}


}  // namespace rmvs
