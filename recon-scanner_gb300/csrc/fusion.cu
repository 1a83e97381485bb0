// fusion.cu -- geometric consistency, voxel fusion, undistortion, scans.
//
// FuseDepthMaps (patchmatch_stereo.cpp:985-1089) accumulates, per voxel
// key, FP64 sums in (map, row, column) order.  Floating-point sums depend
// on order, so the GPU fusion keeps it: points are keyed in FP64 with the
// reference's operation order (bit-identical keys), grouped through a
// device hash table, bucketed per voxel, each bucket sorted back into
// (map, row, column) order and summed sequentially -- the fused cloud is
// bit-identical to the reference's.  Voxels are emitted in order of their
// first point (a deterministic order; the reference's unordered_map order
// is not specified).
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.h"

namespace rmvs {

// Empty-slot key: the table is cleared with a byte memset of 0x7F, so the
// sentinel must be that byte pattern.  A real voxel key can equal it (the
// reference's key is a plain XOR of products): that one key never enters the
// probed table and takes the reserved side slot `mask + 1` instead, so a
// claimed slot is never mistaken for an empty one.
constexpr unsigned long long kEmptyKey = 0x7F7F7F7F7F7F7F7Full;

// ---------------------------------------------------------------------------
// FP64 helpers in the reference's evaluation order (linalg.h:224-232)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mat_t_vec_d(const double* m, const double* v, double* out) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s = __dadd_rn(s, __dmul_rn(m[j * 3 + i], v[j]));
    out[i] = s;
  }
}

__device__ __forceinline__ double norm3_d(const double* v) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s = __dadd_rn(s, __dmul_rn(v[i], v[i]));
  return __dsqrt_rn(s);
}

// Phase 1: per pixel of map m, the reference's filters and FP64 point.
// BgraToGray (orchestrator.cpp:53-67): (77 R + 150 G + 29 B) >> 8, integer.
__global__ void k_bgra_to_gray(const uint8_t* __restrict__ bgra, int w, int h, uint8_t* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  const uchar4 p = reinterpret_cast<const uchar4*>(bgra)[(size_t)y * w + x];
  out[(size_t)y * w + x] = (uint8_t)((77 * (int)p.z + 150 * (int)p.y + 29 * (int)p.x) >> 8);
}

cudaError_t launch_bgra_to_gray(const uint8_t* bgra, int w, int h, uint8_t* out, cudaStream_t st) {
  const dim3 b(32, 8);
  k_bgra_to_gray<<<dim3((w + 31) / 32, (h + 7) / 8), b, 0, st>>>(bgra, w, h, out);
  return cudaGetLastError();
}

__global__ void k_fuse_points(FuseMap M, int64_t base, FuseParams P, unsigned long long* key, double* pos,
                              double* nrm, float* confv, uint8_t* valid) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= M.w || y >= M.h) return;
  const int idx = y * M.w + x;
  const int64_t g = base + idx;
  valid[g] = 0;
  const float depth = M.depth[idx];
  if (!isfinite(depth)) return;
  if ((int)M.support[idx] < P.min_view_consistency) return;
  if (P.photo_threshold < 1.0) {
    const float photo_cost = __fsub_rn(1.0f, M.conf[idx]);
    if ((double)photo_cost > P.photo_threshold) return;
  }
  if (M.keep && !M.keep[idx]) return;
  double ray[3];
  {
    const double xn = __ddiv_rn(__dsub_rn(x + 0.5, M.cx), M.fx);
    const double yn = __ddiv_rn(__dsub_rn(y + 0.5, M.cy), M.fy);
    remove_distortion_d(M.k1, M.k2, M.k3, M.p1, M.p2, xn, yn, &ray[0], &ray[1]);
    ray[2] = 1.0;
  }
  const double d = (double)depth;
  double pc[3], pw[3], nr[3];
  for (int i = 0; i < 3; ++i) pc[i] = __dsub_rn(__dmul_rn(ray[i], d), M.t[i]);
  mat_t_vec_d(M.R, pc, pw);
  double nw[3];
  if (M.normal) {
    // the pixel's plane normal (camera frame, facing the camera) to world
    const double nc[3] = {(double)M.normal[3 * idx], (double)M.normal[3 * idx + 1], (double)M.normal[3 * idx + 2]};
    mat_t_vec_d(M.R, nc, nr);
    const double nn = norm3_d(nr);
    for (int i = 0; i < 3; ++i) nw[i] = nn < 1e-15 ? 0.0 : -__ddiv_rn(nr[i], nn);  // negated below
  } else {
    mat_t_vec_d(M.R, ray, nr);
    const double nn = norm3_d(nr);
    for (int i = 0; i < 3; ++i) nw[i] = nn < 1e-15 ? 0.0 : __ddiv_rn(nr[i], nn);
  }
  const long long vx = (long long)floor(__ddiv_rn(pw[0], P.voxel));
  const long long vy = (long long)floor(__ddiv_rn(pw[1], P.voxel));
  const long long vz = (long long)floor(__ddiv_rn(pw[2], P.voxel));
  const unsigned long long k = ((unsigned long long)vx * 73856093ull) ^ ((unsigned long long)vy * 19349663ull) ^
                               ((unsigned long long)vz * 83492791ull);
  key[g] = k;
  for (int i = 0; i < 3; ++i) {
    pos[3 * g + i] = pw[i];
    nrm[3 * g + i] = -nw[i];
  }
  confv[g] = M.conf[idx];
  valid[g] = 1;
}

__device__ __forceinline__ unsigned long long hash64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

// Phase 2: hash insert; per slot count and first point index.  table_key has
// mask + 1 slots; table_count / table_first have one more, the side slot of
// the key equal to kEmptyKey.
__global__ void k_fuse_insert(int64_t n, const unsigned long long* __restrict__ key, const uint8_t* __restrict__ valid,
                              unsigned long long* table_key, unsigned int* table_count,
                              unsigned long long* table_first, uint64_t mask, int* slot_of, int* error) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n || !valid[g]) return;
  const unsigned long long k = key[g];
  if (k == kEmptyKey) {
    const uint64_t side = mask + 1;
    atomicAdd(&table_count[side], 1u);
    atomicMin(&table_first[side], (unsigned long long)g);
    slot_of[g] = (int)side;
    return;
  }
  uint64_t s = hash64(k) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    const unsigned long long prev = atomicCAS(&table_key[s], kEmptyKey, k);
    if (prev == kEmptyKey || prev == k) {
      atomicAdd(&table_count[s], 1u);
      atomicMin(&table_first[s], (unsigned long long)g);
      slot_of[g] = (int)s;
      return;
    }
    s = (s + 1) & mask;
  }
  slot_of[g] = -1;
  atomicExch(error, 1);
}

// Phase 3: first-occurrence flags (voxel emission order).
__global__ void k_fuse_flags(int64_t n, const uint8_t* __restrict__ valid, const int* __restrict__ slot_of,
                             const unsigned long long* __restrict__ table_first, unsigned int* flag) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int s = slot_of[g];
  flag[g] = (valid[g] && s >= 0 && table_first[s] == (unsigned long long)g) ? 1u : 0u;
}

__global__ void k_fuse_voxels(int64_t n, const unsigned int* __restrict__ flag, const unsigned int* __restrict__ vid_of,
                              const int* __restrict__ slot_of, const unsigned int* __restrict__ table_count,
                              unsigned int* slot_vid, unsigned int* vcount) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n || !flag[g]) return;
  const int s = slot_of[g];
  const unsigned int v = vid_of[g];
  slot_vid[s] = v;
  vcount[v] = table_count[s];
}

__global__ void k_fuse_scatter(int64_t n, const uint8_t* __restrict__ valid, const int* __restrict__ slot_of,
                               const unsigned int* __restrict__ slot_vid, const unsigned int* __restrict__ voffset,
                               unsigned int* cursor, int64_t* bucket) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n || !valid[g] || slot_of[g] < 0) return;
  const unsigned int v = slot_vid[slot_of[g]];
  const unsigned int p = atomicAdd(&cursor[v], 1u);
  bucket[voffset[v] + p] = g;
}

// Phase 6: per voxel, restore (map, row, column) order and sum in it.
__global__ void k_fuse_reduce(unsigned int nvox, const unsigned int* __restrict__ voffset,
                              const unsigned int* __restrict__ vcount, int64_t* bucket,
                              const unsigned long long* __restrict__ key, const double* __restrict__ pos,
                              const double* __restrict__ nrm, const float* __restrict__ confv,
                              unsigned long long* out_key, double* out_pos, double* out_nrm, float* out_conf,
                              unsigned int* out_count) {
  const unsigned int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvox) return;
  int64_t* b = bucket + voffset[v];
  const int cnt = (int)vcount[v];
  // Shell sort (gaps 1, 4, 13, 40, ...) of the point indices
  int gap = 1;
  while (gap < cnt / 3) gap = 3 * gap + 1;
  for (; gap > 0; gap /= 3)
    for (int i = gap; i < cnt; ++i) {
      const int64_t t = b[i];
      int j = i;
      while (j >= gap && b[j - gap] > t) {
        b[j] = b[j - gap];
        j -= gap;
      }
      b[j] = t;
    }
  double sp[3] = {0.0, 0.0, 0.0}, sn[3] = {0.0, 0.0, 0.0}, sc = 0.0;
  for (int i = 0; i < cnt; ++i) {
    const int64_t g = b[i];
    for (int q = 0; q < 3; ++q) sp[q] = __dadd_rn(sp[q], pos[3 * g + q]);
    for (int q = 0; q < 3; ++q) sn[q] = __dadd_rn(sn[q], nrm[3 * g + q]);
    sc = __dadd_rn(sc, (double)confv[g]);
  }
  const double c = (double)cnt;
  for (int q = 0; q < 3; ++q) out_pos[3 * (size_t)v + q] = __ddiv_rn(sp[q], c);
  const double nn = norm3_d(sn);
  if (nn > 1e-12) {
    for (int q = 0; q < 3; ++q) out_nrm[3 * (size_t)v + q] = __ddiv_rn(sn[q], nn);
  } else {
    out_nrm[3 * (size_t)v + 0] = 0.0;
    out_nrm[3 * (size_t)v + 1] = 0.0;
    out_nrm[3 * (size_t)v + 2] = 1.0;
  }
  const double ce = __dmul_rn(__ddiv_rn(sc, c), __dsqrt_rn(c));
  out_conf[v] = (float)(ce < 1.0 ? ce : 1.0);
  out_count[v] = (unsigned int)cnt;
  out_key[v] = key[b[0]];
}

// ---------------------------------------------------------------------------
// geometric consistency (FP32, IEEE operations in a fixed order; the oracle
// performs the identical sequence, so support counts compare bit-exactly)
// ---------------------------------------------------------------------------
__global__ void k_consistency(ConsistencyRef R, const ConsistencySrc* __restrict__ S, int num_src, float rel_max,
                              float reproj2_max, int min_views, uint8_t* out_count, uint8_t* out_keep) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= R.w || y >= R.h) return;
  const int idx = y * R.w + x;
  const float z = R.depth[idx];
  int count = 0;
  const bool zok = z > 0.0f && isfinite(z);
  if (zok) {
    const float xr = __fdiv_rn(__fsub_rn(__fadd_rn((float)x, 0.5f), R.cx), R.fx);
    const float yr = __fdiv_rn(__fsub_rn(__fadd_rn((float)y, 0.5f), R.cy), R.fy);
    const float P0 = __fmul_rn(xr, z), P1 = __fmul_rn(yr, z), P2 = z;
    for (int s = 0; s < num_src; ++s) {
      const ConsistencySrc& C = S[s];
      const float* A = C.A;
      const float* b = C.b;
      const float Q0 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(A[0], P0), __fmul_rn(A[1], P1)), __fmul_rn(A[2], P2)), b[0]);
      const float Q1 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(A[3], P0), __fmul_rn(A[4], P1)), __fmul_rn(A[5], P2)), b[1]);
      const float Q2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(A[6], P0), __fmul_rn(A[7], P1)), __fmul_rn(A[8], P2)), b[2]);
      if (!(Q2 > 1e-6f)) continue;
      const float us = __fadd_rn(__fmul_rn(C.fx, __fdiv_rn(Q0, Q2)), C.cx);
      const float vs = __fadd_rn(__fmul_rn(C.fy, __fdiv_rn(Q1, Q2)), C.cy);
      if (!(us >= 0.0f && us < (float)C.w && vs >= 0.0f && vs < (float)C.h)) continue;
      const int ix = (int)us, iy = (int)vs;
      const float zs = C.depth[(size_t)iy * C.w + ix];
      if (!(zs > 0.0f) || !isfinite(zs)) continue;
      const float xs = __fdiv_rn(__fsub_rn(__fadd_rn((float)ix, 0.5f), C.cx), C.fx);
      const float ys = __fdiv_rn(__fsub_rn(__fadd_rn((float)iy, 0.5f), C.cy), C.fy);
      const float S0 = __fmul_rn(xs, zs), S1 = __fmul_rn(ys, zs), S2 = zs;
      const float* Ai = C.Ai;
      const float* bi = C.bi;
      const float B0 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(Ai[0], S0), __fmul_rn(Ai[1], S1)), __fmul_rn(Ai[2], S2)), bi[0]);
      const float B1 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(Ai[3], S0), __fmul_rn(Ai[4], S1)), __fmul_rn(Ai[5], S2)), bi[1]);
      const float B2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(Ai[6], S0), __fmul_rn(Ai[7], S1)), __fmul_rn(Ai[8], S2)), bi[2]);
      if (!(B2 > 1e-6f)) continue;
      const float rel = __fdiv_rn(fabsf(__fsub_rn(B2, z)), z);
      const float ur = __fadd_rn(__fmul_rn(R.fx, __fdiv_rn(B0, B2)), R.cx);
      const float vr = __fadd_rn(__fmul_rn(R.fy, __fdiv_rn(B1, B2)), R.cy);
      const float du = __fsub_rn(ur, __fadd_rn((float)x, 0.5f));
      const float dv = __fsub_rn(vr, __fadd_rn((float)y, 0.5f));
      const float e2 = __fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv));
      if (rel <= rel_max && e2 <= reproj2_max) ++count;
    }
  }
  out_count[idx] = (uint8_t)min(count, 255);
  out_keep[idx] = (uint8_t)(zok && count >= min_views);
}

// ---------------------------------------------------------------------------
// undistortion: output pixel centre -> ApplyDistortion (camera.cpp:33-45) ->
// bilinear read with the pixel-centre convention, FP64, 0 outside
// ---------------------------------------------------------------------------
__global__ void k_undistort(const uint8_t* __restrict__ img, int w, int h, UndistortCam K, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= w || j >= h) return;
  const double xn = __ddiv_rn(__dsub_rn(i + 0.5, K.cx), K.fx);
  const double yn = __ddiv_rn(__dsub_rn(j + 0.5, K.cy), K.fy);
  double xd, yd;
  apply_distortion_d(K.k1, K.k2, K.k3, K.p1, K.p2, xn, yn, &xd, &yd);
  const double u = __dsub_rn(__dadd_rn(__dmul_rn(K.fx, xd), K.cx), 0.5);
  const double v = __dsub_rn(__dadd_rn(__dmul_rn(K.fy, yd), K.cy), 0.5);
  double val = 0.0;
  if (!(u < 0.0 || v < 0.0 || u > (double)(w - 1) || v > (double)(h - 1))) {
    const int x0 = (int)floor(u), y0 = (int)floor(v);
    const int x1 = min(x0 + 1, w - 1), y1 = min(y0 + 1, h - 1);
    const double fx = __dsub_rn(u, (double)x0), fy = __dsub_rn(v, (double)y0);
    const double p00 = img[y0 * w + x0], p10 = img[y0 * w + x1], p01 = img[y1 * w + x0], p11 = img[y1 * w + x1];
    const double top = __dadd_rn(__dmul_rn(p00, __dsub_rn(1.0, fx)), __dmul_rn(p10, fx));
    const double bot = __dadd_rn(__dmul_rn(p01, __dsub_rn(1.0, fx)), __dmul_rn(p11, fx));
    val = __dadd_rn(__dmul_rn(top, __dsub_rn(1.0, fy)), __dmul_rn(bot, fy));
  }
  out[(size_t)j * w + i] = (float)val;
}

// ---------------------------------------------------------------------------
// 3x3 binomial low-pass ([1 2 1]/4 in each direction, edge-clamped): the
// optional staging pre-filter.  Input u8 (in_u8) or float (in_f32).
// ---------------------------------------------------------------------------
__global__ void k_binomial(const uint8_t* __restrict__ in_u8, const float* __restrict__ in_f32, int w, int h,
                           float* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w || y >= h) return;
  float acc = 0.f;
#pragma unroll
  for (int j = -1; j <= 1; ++j) {
    const int yy = min(max(y + j, 0), h - 1);
    const float wy = j == 0 ? 0.5f : 0.25f;
#pragma unroll
    for (int i = -1; i <= 1; ++i) {
      const int xx = min(max(x + i, 0), w - 1);
      const float wx = i == 0 ? 0.5f : 0.25f;
      const float v = in_u8 ? (float)in_u8[(size_t)yy * w + xx] : in_f32[(size_t)yy * w + xx];
      acc = fmaf(wx * wy, v, acc);
    }
  }
  out[(size_t)y * w + x] = acc;
}

// Pyramid level 1: each pixel the mean of a 2 x 2 block of the staged image
// (8-bit or FP32), so that level-1 pixel centre i + 0.5 is level-0
// coordinate 2 i + 1 (focal lengths and principal point halve).
__global__ void k_half_level(const uint8_t* __restrict__ in_u8, const float* __restrict__ in_f32, int w, int h,
                             int w1, int h1, float* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= w1 || y >= h1) return;
  const size_t i0 = (size_t)(2 * y) * w + 2 * x, i1 = i0 + w;
  float a, b, c, d;
  if (in_u8) {
    a = in_u8[i0];
    b = in_u8[i0 + 1];
    c = in_u8[i1];
    d = in_u8[i1 + 1];
  } else {
    a = in_f32[i0];
    b = in_f32[i0 + 1];
    c = in_f32[i1];
    d = in_f32[i1 + 1];
  }
  out[(size_t)y * w1 + x] = 0.25f * ((a + b) + (c + d));
}

cudaError_t launch_half_level(const uint8_t* in_u8, const float* in_f32, int w, int h, float* out, cudaStream_t st) {
  const int w1 = w / 2, h1 = h / 2;
  if (w1 < 1 || h1 < 1) return cudaErrorInvalidValue;
  const dim3 b(32, 8);
  k_half_level<<<dim3((w1 + 31) / 32, (h1 + 7) / 8), b, 0, st>>>(in_u8, in_f32, w, h, w1, h1, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// exclusive scan of uint32 (three-phase, recursive over block sums)
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;

__global__ void k_scan_block(const unsigned int* in, unsigned int* out, int64_t n, unsigned int* block_sums) {
  __shared__ unsigned int s[kScanBlock];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock;
  const int t = threadIdx.x;
  const unsigned int v = (base + t < n) ? in[base + t] : 0u;
  s[t] = v;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    const unsigned int a = t >= off ? s[t - off] : 0u;
    __syncthreads();
    s[t] += a;
    __syncthreads();
  }
  if (base + t < n) out[base + t] = s[t] - v;
  if (t == kScanBlock - 1) block_sums[blockIdx.x] = s[t];
}

__global__ void k_scan_add(unsigned int* out, int64_t n, const unsigned int* block_offsets) {
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += block_offsets[blockIdx.x];
}

// scratch: at least scan_scratch_elems(n) uint32
int64_t scan_scratch_elems(int64_t n) {
  int64_t total = 0;
  while (n > 1) {
    n = (n + kScanBlock - 1) / kScanBlock;
    total += 2 * n;
  }
  return total + 2;
}

cudaError_t exclusive_scan_u32(const unsigned int* in, unsigned int* out, int64_t n, unsigned int* scratch,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  unsigned int* sums = scratch;
  unsigned int* offs = scratch + nb;
  k_scan_block<<<(unsigned)nb, kScanBlock, 0, st>>>(in, out, n, sums);
  if (nb > 1) {
    cudaError_t e = exclusive_scan_u32(sums, offs, nb, scratch + 2 * nb, st);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, st>>>(out, n, offs);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static dim3 g2(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }
static unsigned b1(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t launch_fuse_points(const FuseMap& M, int64_t base, const FuseParams& P, unsigned long long* key,
                               double* pos, double* nrm, float* conf, uint8_t* valid, cudaStream_t st) {
  const dim3 b(32, 8);
  k_fuse_points<<<g2(M.w, M.h, b), b, 0, st>>>(M, base, P, key, pos, nrm, conf, valid);
  return cudaGetLastError();
}

cudaError_t launch_fuse_insert(int64_t n, const unsigned long long* key, const uint8_t* valid,
                               unsigned long long* tkey, unsigned int* tcount, unsigned long long* tfirst,
                               uint64_t mask, int* slot_of, int* error, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_fuse_insert<<<b1(n, 256), 256, 0, st>>>(n, key, valid, tkey, tcount, tfirst, mask, slot_of, error);
  return cudaGetLastError();
}

cudaError_t launch_fuse_flags(int64_t n, const uint8_t* valid, const int* slot_of, const unsigned long long* tfirst,
                              unsigned int* flag, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_fuse_flags<<<b1(n, 256), 256, 0, st>>>(n, valid, slot_of, tfirst, flag);
  return cudaGetLastError();
}

cudaError_t launch_fuse_voxels(int64_t n, const unsigned int* flag, const unsigned int* vid_of, const int* slot_of,
                               const unsigned int* tcount, unsigned int* slot_vid, unsigned int* vcount,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_fuse_voxels<<<b1(n, 256), 256, 0, st>>>(n, flag, vid_of, slot_of, tcount, slot_vid, vcount);
  return cudaGetLastError();
}

cudaError_t launch_fuse_scatter(int64_t n, const uint8_t* valid, const int* slot_of, const unsigned int* slot_vid,
                                const unsigned int* voffset, unsigned int* cursor, int64_t* bucket, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_fuse_scatter<<<b1(n, 256), 256, 0, st>>>(n, valid, slot_of, slot_vid, voffset, cursor, bucket);
  return cudaGetLastError();
}

cudaError_t launch_fuse_reduce(unsigned int nvox, const unsigned int* voffset, const unsigned int* vcount,
                               int64_t* bucket, const unsigned long long* key, const double* pos, const double* nrm,
                               const float* conf, unsigned long long* okey, double* opos, double* onrm, float* oconf,
                               unsigned int* ocount, cudaStream_t st) {
  if (nvox == 0) return cudaSuccess;
  k_fuse_reduce<<<b1(nvox, 128), 128, 0, st>>>(nvox, voffset, vcount, bucket, key, pos, nrm, conf, okey, opos, onrm,
                                               oconf, ocount);
  return cudaGetLastError();
}

// A fused cloud's Poisson point weights max(0, confidence) and the bounds of
// its positions (min x, y, z, max x, y, z), one block: the order of the
// min / max reduction does not change its result.
constexpr int kBoundsThreads = 512;
__global__ void __launch_bounds__(kBoundsThreads) k_cloud_finish(const double* __restrict__ pos,
                                                                 const float* __restrict__ conf, unsigned int n,
                                                                 float* weights, double* bounds) {
  __shared__ double red[6][kBoundsThreads];
  double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
  for (unsigned int i = threadIdx.x; i < n; i += kBoundsThreads) {
    weights[i] = fmaxf(0.0f, conf[i]);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double v = pos[3 * (size_t)i + q];
      lo[q] = fmin(lo[q], v);
      hi[q] = fmax(hi[q], v);
    }
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    red[q][threadIdx.x] = lo[q];
    red[3 + q][threadIdx.x] = hi[q];
  }
  __syncthreads();
  for (int off = kBoundsThreads / 2; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        red[q][threadIdx.x] = fmin(red[q][threadIdx.x], red[q][threadIdx.x + off]);
        red[3 + q][threadIdx.x] = fmax(red[3 + q][threadIdx.x], red[3 + q][threadIdx.x + off]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) bounds[threadIdx.x] = red[threadIdx.x][0];
}

cudaError_t launch_cloud_finish(const double* pos, const float* conf, unsigned int n, float* weights, double* bounds,
                                cudaStream_t st) {
  k_cloud_finish<<<1, kBoundsThreads, 0, st>>>(pos, conf, n, weights, bounds);
  return cudaGetLastError();
}

cudaError_t launch_consistency(const ConsistencyRef& R, const ConsistencySrc* S, int num_src, float rel_max,
                               float reproj_px_max, int min_views, uint8_t* count, uint8_t* keep, cudaStream_t st) {
  const dim3 b(32, 8);
  const float r2 = reproj_px_max * reproj_px_max;
  k_consistency<<<g2(R.w, R.h, b), b, 0, st>>>(R, S, num_src, rel_max, r2, min_views, count, keep);
  return cudaGetLastError();
}

cudaError_t launch_binomial(const uint8_t* in_u8, const float* in_f32, int w, int h, float* out, cudaStream_t st) {
  const dim3 b(32, 8);
  k_binomial<<<g2(w, h, b), b, 0, st>>>(in_u8, in_f32, w, h, out);
  return cudaGetLastError();
}

cudaError_t launch_undistort(const uint8_t* img, int w, int h, const UndistortCam& K, float* out, cudaStream_t st) {
  const dim3 b(32, 8);
  k_undistort<<<g2(w, h, b), b, 0, st>>>(img, w, h, K, out);
  return cudaGetLastError();
}

}  // namespace rmvs
