// tsdf.cu -- TSDF fusion of depth frames into a device-resident voxel grid.
//
// The reference's TsdfVolume (core/src/rgbd/tsdf_fusion.cpp with the shared
// kernel core/src/rgbd/tsdf_internal.h) walks each valid pixel's viewing ray
// across the truncation band and folds every voxel it meets into a running
// weighted mean, pixel after pixel in raster order.  A voxel can be met by
// many pixels of one frame, and floating-point running means depend on their
// order, so the GPU keeps it: every (pixel, step) pair becomes one update
// record whose index is its place in the reference's order; records are
// counted per voxel, bucketed, each bucket sorted back into record order and
// folded in sequence by one thread per voxel.  The grid -- and the surface
// points extracted from it -- are bit-identical to the reference's.  All FP64
// and FP32 arithmetic is written with explicit round-to-nearest operations
// in the reference's evaluation order (no contractions).
//
// Layout in HBM: tsdf and weight as FP32 arrays over the dense grid, index
// (iz * ny + iy) * nx + ix, as in the reference (8 bytes per voxel; the
// reference also keeps 12 bytes of colour it never writes).
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "kernels.h"
#include "recon_mvs_gb300.h"

namespace rmvs {

extern thread_local std::string g_last_error;

namespace {

struct TsdfFrame {
  int w, h;
  int nx, ny, nz;
  int steps;
  float voxel, trunc, w_new;
  double fx, fy, cx, cy, min_depth, max_depth;
  int min_conf;
  double origin[3];
  double R_wc[9], t_wc[3], R_cw[9], t_cw[3];
};

__device__ __forceinline__ void mat3_vec_rn(const double* m, const double* v, double* out) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) s = __dadd_rn(s, __dmul_rn(m[i * 3 + j], v[j]));
    out[i] = s;
  }
}

__device__ __forceinline__ void normalized_rn(const double* v, double* out) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) s = __dadd_rn(s, __dmul_rn(v[i], v[i]));
  const double n = __dsqrt_rn(s);
  if (n < 1e-15) {
    out[0] = out[1] = out[2] = 0.0;
    return;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) out[i] = __ddiv_rn(v[i], n);
}

__device__ __forceinline__ int floor_scaled(float a, float b) { return (int)floorf(__fdiv_rn(a, b)); }

// One thread per pixel: the pixel's update records, one per step of its
// ray walk (record index = pixel * (2 steps + 1) + step: the reference's
// update order), voxel index -1 where the step writes nothing.
__global__ void k_tsdf_records(TsdfFrame F, const uint16_t* __restrict__ depth, const uint8_t* __restrict__ conf,
                               int* rec_vox, float* rec_sdf, unsigned int* integrated) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y * blockDim.y + threadIdx.y;
  if (u >= F.w || v >= F.h) return;
  const size_t pix = (size_t)v * F.w + u;
  const int nst = 2 * F.steps + 1;
  int* rv = rec_vox + pix * nst;
  for (int k = 0; k < nst; ++k) rv[k] = -1;
  const uint16_t d_raw = depth[pix];
  if (d_raw == 0) return;
  if (conf && (int)conf[pix] < F.min_conf) return;
  const double dx = __ddiv_rn(__dsub_rn((double)u, F.cx), F.fx);
  const double dy = __ddiv_rn(__dsub_rn((double)v, F.cy), F.fy);
  const double d = __dmul_rn((double)d_raw, 1e-3);
  if (d < F.min_depth || d > F.max_depth) return;
  atomicAdd(integrated, 1u);
  const double p_cam[3] = {__dmul_rn(dx, d), __dmul_rn(dy, d), d};
  double pw[3], ray[3], rw[3], nw[3];
  mat3_vec_rn(F.R_cw, p_cam, pw);
#pragma unroll
  for (int i = 0; i < 3; ++i) pw[i] = __dadd_rn(pw[i], F.t_cw[i]);
  normalized_rn(p_cam, ray);
  mat3_vec_rn(F.R_cw, ray, rw);
  normalized_rn(rw, nw);
  const int cxv = floor_scaled(__double2float_rn(__dsub_rn(pw[0], F.origin[0])), F.voxel);
  const int cyv = floor_scaled(__double2float_rn(__dsub_rn(pw[1], F.origin[1])), F.voxel);
  const int czv = floor_scaled(__double2float_rn(__dsub_rn(pw[2], F.origin[2])), F.voxel);
  const float nxw = __double2float_rn(nw[0]), nyw = __double2float_rn(nw[1]), nzw = __double2float_rn(nw[2]);
  const float ox = __double2float_rn(F.origin[0]), oy = __double2float_rn(F.origin[1]),
              oz = __double2float_rn(F.origin[2]);
  const double trunc = (double)F.trunc;
  float* rs = rec_sdf + pix * nst;
  for (int s = -F.steps; s <= F.steps; ++s) {
    const float dist = __fmul_rn((float)s, F.voxel);
    const int ix = cxv + floor_scaled(__fmul_rn(dist, nxw), F.voxel);
    const int iy = cyv + floor_scaled(__fmul_rn(dist, nyw), F.voxel);
    const int iz = czv + floor_scaled(__fmul_rn(dist, nzw), F.voxel);
    if (!(ix >= 0 && iy >= 0 && iz >= 0 && ix < F.nx && iy < F.ny && iz < F.nz)) continue;
    const double vw[3] = {(double)__fadd_rn(ox, __fmul_rn(__fadd_rn((float)ix, 0.5f), F.voxel)),
                          (double)__fadd_rn(oy, __fmul_rn(__fadd_rn((float)iy, 0.5f), F.voxel)),
                          (double)__fadd_rn(oz, __fmul_rn(__fadd_rn((float)iz, 0.5f), F.voxel))};
    double vc[3];
    mat3_vec_rn(F.R_wc, vw, vc);
#pragma unroll
    for (int i = 0; i < 3; ++i) vc[i] = __dadd_rn(vc[i], F.t_wc[i]);
    if (vc[2] <= 1e-6) continue;
    const long long pxi = llround(__dadd_rn(__ddiv_rn(__dmul_rn(F.fx, vc[0]), vc[2]), F.cx));
    const long long pyi = llround(__dadd_rn(__ddiv_rn(__dmul_rn(F.fy, vc[1]), vc[2]), F.cy));
    if (pxi < 0 || pxi >= F.w || pyi < 0 || pyi >= F.h) continue;
    const double diff = __dsub_rn(d, vc[2]);
    if (fabs(diff) > trunc) continue;
    rv[s + F.steps] = (iz * F.ny + iy) * F.nx + ix;
    rs[s + F.steps] = __double2float_rn(__ddiv_rn(diff, trunc));
  }
}

__global__ void k_tsdf_count(const int* __restrict__ rec_vox, int64_t n, unsigned int* count) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int vx = rec_vox[r];
  if (vx >= 0) atomicAdd(&count[vx], 1u);
}

__global__ void k_tsdf_scatter(const int* __restrict__ rec_vox, int64_t n, const unsigned int* __restrict__ offset,
                               unsigned int* cursor, unsigned int* bucket) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int vx = rec_vox[r];
  if (vx < 0) return;
  bucket[offset[vx] + atomicAdd(&cursor[vx], 1u)] = (unsigned int)r;
}

// One thread per voxel: its records back in the reference's order, folded
// into the running weighted mean (tsdf_fusion.cpp:95-102).
__global__ void k_tsdf_apply(int64_t nvox, const unsigned int* __restrict__ count,
                             const unsigned int* __restrict__ offset, unsigned int* bucket,
                             const float* __restrict__ rec_sdf, float w_new, float* tsdf, float* weight) {
  const int64_t vx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (vx >= nvox) return;
  const int c = (int)count[vx];
  if (c == 0) return;
  unsigned int* b = bucket + offset[vx];
  for (int i = 1; i < c; ++i) {  // insertion sort: buckets hold a few records
    const unsigned int t = b[i];
    int j = i;
    while (j > 0 && b[j - 1] > t) {
      b[j] = b[j - 1];
      --j;
    }
    b[j] = t;
  }
  float t = tsdf[vx], w = weight[vx];
  for (int i = 0; i < c; ++i) {
    const float sdf = rec_sdf[b[i]];
    const float w_sum = __fadd_rn(w, w_new);
    if (w_sum > 0.0f) {
      t = __fdiv_rn(__fadd_rn(__fmul_rn(w, t), __fmul_rn(w_new, sdf)), w_sum);
      w = w_sum;
    }
  }
  tsdf[vx] = t;
  weight[vx] = w;
}

__global__ void k_tsdf_fill(int64_t n, float* tsdf, float* weight) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  tsdf[i] = 1.0f;
  weight[i] = 0.0f;
}

// SurfaceGradient (tsdf_internal.h:154-187) at voxel (ix, iy, iz).
__device__ bool surface_gradient(const float* __restrict__ tsdf, const float* __restrict__ weight, int nx, int ny,
                                 int nz, int ix, int iy, int iz, float* onx, float* ony, float* onz) {
  const size_t i0 = ((size_t)iz * ny + iy) * nx + ix;
  if (weight[i0] <= 0.0f) return false;  // never fused
  if (tsdf[i0] > 0.0f) return false;
  const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  bool pos = false;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int a = ix + off[k][0], b = iy + off[k][1], c = iz + off[k][2];
    if (!(a >= 0 && b >= 0 && c >= 0 && a < nx && b < ny && c < nz)) continue;
    const size_t j = ((size_t)c * ny + b) * nx + a;
    if (weight[j] > 0.0f && tsdf[j] > 0.0f) {
      pos = true;
      sx = __fadd_rn(sx, (float)off[k][0]);
      sy = __fadd_rn(sy, (float)off[k][1]);
      sz = __fadd_rn(sz, (float)off[k][2]);
    }
  }
  if (!pos) return false;
  const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(sx, sx), __fmul_rn(sy, sy)), __fmul_rn(sz, sz)));
  if (len < 1e-9f) return false;
  *onx = __fdiv_rn(sx, len);
  *ony = __fdiv_rn(sy, len);
  *onz = __fdiv_rn(sz, len);
  return true;
}

__global__ void k_tsdf_surface_flags(const float* __restrict__ tsdf, const float* __restrict__ weight, int nx, int ny,
                                     int nz, unsigned int* flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)nx * ny * nz;
  if (i >= n) return;
  const int ix = (int)(i % nx), iy = (int)((i / nx) % ny), iz = (int)(i / ((int64_t)nx * ny));
  float a, b, c;
  flag[i] = surface_gradient(tsdf, weight, nx, ny, nz, ix, iy, iz, &a, &b, &c) ? 1u : 0u;
}

// ExtractPoints (tsdf_fusion.cpp:106-140) in (iz, iy, ix) order: the
// surface voxels' centres (VoxelToWorld: FP64 origin + FP32 offset, rounded
// to FP32), normals, confidences min(1, weight / 64).
__global__ void k_tsdf_surface_emit(const float* __restrict__ tsdf, const float* __restrict__ weight, int nx, int ny,
                                    int nz, const unsigned int* __restrict__ flag,
                                    const unsigned int* __restrict__ slot, double ox, double oy, double oz,
                                    float voxel, double* pos, double* nrm, float* conf, int64_t* key) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)nx * ny * nz;
  if (i >= n || !flag[i]) return;
  const int ix = (int)(i % nx), iy = (int)((i / nx) % ny), iz = (int)(i / ((int64_t)nx * ny));
  float a, b, c;
  surface_gradient(tsdf, weight, nx, ny, nz, ix, iy, iz, &a, &b, &c);
  const unsigned int k = slot[i];
  pos[3 * (size_t)k + 0] = (double)__double2float_rn(__dadd_rn(ox, (double)__fmul_rn(__fadd_rn((float)ix, 0.5f), voxel)));
  pos[3 * (size_t)k + 1] = (double)__double2float_rn(__dadd_rn(oy, (double)__fmul_rn(__fadd_rn((float)iy, 0.5f), voxel)));
  pos[3 * (size_t)k + 2] = (double)__double2float_rn(__dadd_rn(oz, (double)__fmul_rn(__fadd_rn((float)iz, 0.5f), voxel)));
  nrm[3 * (size_t)k + 0] = (double)a;
  nrm[3 * (size_t)k + 1] = (double)b;
  nrm[3 * (size_t)k + 2] = (double)c;
  conf[k] = fminf(1.0f, __fdiv_rn(weight[i], 64.0f));
  key[k] = i;
}

// Device buffer that grows on demand.
template <class T>
struct TBuf {
  T* p = nullptr;
  size_t n = 0;
  ~TBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    const cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
};

// FloorToIntScaled of the bounding-box extent + 1 (tsdf_fusion.cpp:36-47).
int grid_dim(double bbox_max, float origin, float voxel) {
  const int n = (int)floorf((float)(bbox_max - (double)origin) / voxel) + 1;
  return n > 1 ? n : 1;
}

}  // namespace

struct TsdfVolume {
  recon_tsdf_config cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  int nx = 1, ny = 1, nz = 1;
  int64_t nvox = 1;
  float voxel = 0.0f;
  double origin[3] = {0, 0, 0};
  TBuf<float> tsdf, weight;
  TBuf<uint16_t> depth;
  TBuf<uint8_t> conf;
  TBuf<int> rec_vox;
  TBuf<float> rec_sdf;
  TBuf<unsigned int> count, offset, cursor, bucket, scratch, integrated;
  ~TsdfVolume() {
    cudaSetDevice(device);
    if (stream) cudaStreamDestroy(stream);
  }
};

}  // namespace rmvs

using namespace rmvs;

namespace {

recon_status tsdf_fail(recon_status st, const std::string& what) {
  g_last_error = what;
  return st;
}

recon_status cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();
  g_last_error = std::string("tsdf: ") + what + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? RECON_ERR_OUT_OF_MEMORY : RECON_ERR_MVS_GPU_FAILURE;
}

#define TCK(call, what)                        \
  do {                                         \
    const cudaError_t e_ = (call);             \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" {

RECON_API recon_status recon_tsdf_config_default(recon_tsdf_config* out) {
  if (!out) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_config_default: NULL");
  std::memset(out, 0, sizeof(*out));
  out->voxel_size_m = 0.001;
  out->truncation_m = 0.008;
  out->min_depth_m = 0.05;
  out->max_depth_m = 3.0;
  out->fx = 1.0;
  out->fy = 1.0;
  out->bbox_max_x = 1.0;
  out->bbox_max_y = 1.0;
  out->bbox_max_z = 1.0;
  out->min_confidence = 30;
  return RECON_OK;
}

RECON_API recon_status recon_tsdf_create(const recon_tsdf_config* cfg, int32_t device, void** out_volume) {
  if (!cfg || !out_volume) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_create: NULL argument");
  *out_volume = nullptr;
  if (!(cfg->voxel_size_m > 0.0) || !(cfg->fx != 0.0) || !(cfg->fy != 0.0))
    return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_create: voxel size must be > 0 and focal lengths non-zero");
  auto* V = new (std::nothrow) TsdfVolume();
  if (!V) return tsdf_fail(RECON_ERR_OUT_OF_MEMORY, "tsdf_create: host allocation failed");
  V->cfg = *cfg;
  V->device = device;
  V->voxel = (float)cfg->voxel_size_m;
  V->origin[0] = (double)(float)cfg->origin_x;
  V->origin[1] = (double)(float)cfg->origin_y;
  V->origin[2] = (double)(float)cfg->origin_z;
  V->nx = grid_dim(cfg->bbox_max_x, (float)cfg->origin_x, V->voxel);
  V->ny = grid_dim(cfg->bbox_max_y, (float)cfg->origin_y, V->voxel);
  V->nz = grid_dim(cfg->bbox_max_z, (float)cfg->origin_z, V->voxel);
  V->nvox = (int64_t)V->nx * V->ny * V->nz;
  if (V->nvox >= (int64_t)1 << 31) {
    delete V;
    return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_create: more than 2^31 voxels");
  }
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&V->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = V->tsdf.reserve(V->nvox);
  if (e == cudaSuccess) e = V->weight.reserve(V->nvox);
  if (e == cudaSuccess) {
    k_tsdf_fill<<<blocks_for(V->nvox, 256), 256, 0, V->stream>>>(V->nvox, V->tsdf.p, V->weight.p);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(V->stream);
  if (e != cudaSuccess) {
    const recon_status st = cuda_fail(e, "create");
    delete V;
    return st;
  }
  *out_volume = V;
  g_last_error.clear();
  return RECON_OK;
}

RECON_API recon_status recon_tsdf_integrate(void* volume, const uint16_t* depth_mm, const uint8_t* confidence,
                                            int32_t width, int32_t height, const double* world_to_camera,
                                            float depth_uncertainty_m, uint32_t* out_integrated) {
  if (out_integrated) *out_integrated = 0;
  if (!volume || !world_to_camera) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_integrate: NULL argument");
  TsdfVolume& V = *static_cast<TsdfVolume*>(volume);
  const recon_tsdf_config& c = V.cfg;
  // IntegrateFrame's early returns (tsdf_internal.h:50-54)
  if (!depth_mm || width <= 0 || height <= 0) return RECON_OK;
  const float trunc = (float)c.truncation_m;
  if (V.voxel <= 0.0f || trunc <= 0.0f) return RECON_OK;
  if ((int64_t)width * height > ((int64_t)1 << 26))
    return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_integrate: frame larger than 2^26 pixels");
  TsdfFrame F;
  std::memset(&F, 0, sizeof(F));
  F.w = width;
  F.h = height;
  F.nx = V.nx;
  F.ny = V.ny;
  F.nz = V.nz;
  F.voxel = V.voxel;
  F.trunc = trunc;
  F.steps = (int)(trunc / V.voxel) + 1;
  const double sig = (double)depth_uncertainty_m;
  const double sigma = sig > 1e-4 ? sig : 1e-4;
  F.w_new = (float)(1.0 / (sigma * sigma));
  F.fx = c.fx;
  F.fy = c.fy;
  F.cx = c.cx;
  F.cy = c.cy;
  F.min_depth = c.min_depth_m;
  F.max_depth = c.max_depth_m;
  F.min_conf = c.min_confidence;
  for (int i = 0; i < 3; ++i) F.origin[i] = V.origin[i];
  // R_cw = R_wc^T, t_cw = -(R_cw t_wc) (tsdf_internal.h:57-69), host FP64 in
  // the reference's order (this file is compiled without contractions)
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) F.R_wc[i * 3 + j] = world_to_camera[i * 4 + j];
    F.t_wc[i] = world_to_camera[i * 4 + 3];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) F.R_cw[j * 3 + i] = F.R_wc[i * 3 + j];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += F.R_cw[i * 3 + j] * F.t_wc[j];
    F.t_cw[i] = -s;
  }
  TCK(cudaSetDevice(V.device), "set device");
  const size_t npix = (size_t)width * height;
  const int64_t nrec = (int64_t)npix * (2 * F.steps + 1);
  if (nrec >= ((int64_t)1 << 32)) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_integrate: too many updates");
  TCK(V.depth.reserve(npix), "alloc");
  if (confidence) TCK(V.conf.reserve(npix), "alloc");
  TCK(V.rec_vox.reserve(nrec), "alloc");
  TCK(V.rec_sdf.reserve(nrec), "alloc");
  TCK(V.bucket.reserve(nrec), "alloc");
  TCK(V.count.reserve(V.nvox), "alloc");
  TCK(V.offset.reserve(V.nvox), "alloc");
  TCK(V.cursor.reserve(V.nvox), "alloc");
  TCK(V.scratch.reserve(scan_scratch_elems(V.nvox)), "alloc");
  TCK(V.integrated.reserve(1), "alloc");
  cudaStream_t st = V.stream;
  TCK(cudaMemcpyAsync(V.depth.p, depth_mm, npix * sizeof(uint16_t), cudaMemcpyHostToDevice, st), "upload");
  if (confidence) TCK(cudaMemcpyAsync(V.conf.p, confidence, npix, cudaMemcpyHostToDevice, st), "upload");
  TCK(cudaMemsetAsync(V.integrated.p, 0, sizeof(unsigned int), st), "memset");
  TCK(cudaMemsetAsync(V.count.p, 0, V.nvox * sizeof(unsigned int), st), "memset");
  TCK(cudaMemsetAsync(V.cursor.p, 0, V.nvox * sizeof(unsigned int), st), "memset");
  const dim3 b2(32, 8);
  k_tsdf_records<<<dim3((width + 31) / 32, (height + 7) / 8), b2, 0, st>>>(
      F, V.depth.p, confidence ? V.conf.p : nullptr, V.rec_vox.p, V.rec_sdf.p, V.integrated.p);
  TCK(cudaGetLastError(), "records");
  k_tsdf_count<<<blocks_for(nrec, 256), 256, 0, st>>>(V.rec_vox.p, nrec, V.count.p);
  TCK(cudaGetLastError(), "count");
  TCK(exclusive_scan_u32(V.count.p, V.offset.p, V.nvox, V.scratch.p, st), "scan");
  k_tsdf_scatter<<<blocks_for(nrec, 256), 256, 0, st>>>(V.rec_vox.p, nrec, V.offset.p, V.cursor.p, V.bucket.p);
  TCK(cudaGetLastError(), "scatter");
  k_tsdf_apply<<<blocks_for(V.nvox, 256), 256, 0, st>>>(V.nvox, V.count.p, V.offset.p, V.bucket.p, V.rec_sdf.p,
                                                        F.w_new, V.tsdf.p, V.weight.p);
  TCK(cudaGetLastError(), "apply");
  unsigned int n = 0;
  TCK(cudaMemcpyAsync(&n, V.integrated.p, sizeof(n), cudaMemcpyDeviceToHost, st), "download");
  TCK(cudaStreamSynchronize(st), "integrate");
  if (out_integrated) *out_integrated = n;
  g_last_error.clear();
  return RECON_OK;
}

RECON_API recon_status recon_tsdf_extract_points(void* volume, recon_mvs_point_cloud* out) {
  if (!volume || !out) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_extract_points: NULL argument");
  std::memset(out, 0, sizeof(*out));
  TsdfVolume& V = *static_cast<TsdfVolume*>(volume);
  TCK(cudaSetDevice(V.device), "set device");
  cudaStream_t st = V.stream;
  TBuf<unsigned int> flag, slot;
  TCK(flag.reserve(V.nvox), "alloc");
  TCK(slot.reserve(V.nvox), "alloc");
  TCK(V.scratch.reserve(scan_scratch_elems(V.nvox)), "alloc");
  k_tsdf_surface_flags<<<blocks_for(V.nvox, 256), 256, 0, st>>>(V.tsdf.p, V.weight.p, V.nx, V.ny, V.nz, flag.p);
  TCK(cudaGetLastError(), "flags");
  TCK(exclusive_scan_u32(flag.p, slot.p, V.nvox, V.scratch.p, st), "scan");
  unsigned int last_slot = 0, last_flag = 0;
  TCK(cudaMemcpyAsync(&last_slot, slot.p + V.nvox - 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, st), "download");
  TCK(cudaMemcpyAsync(&last_flag, flag.p + V.nvox - 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, st), "download");
  TCK(cudaStreamSynchronize(st), "extract");
  const size_t n = (size_t)last_slot + last_flag;
  if (n == 0) {
    g_last_error.clear();
    return RECON_OK;
  }
  TBuf<double> pos, nrm;
  TBuf<float> conf;
  TBuf<int64_t> key;
  TCK(pos.reserve(3 * n), "alloc");
  TCK(nrm.reserve(3 * n), "alloc");
  TCK(conf.reserve(n), "alloc");
  TCK(key.reserve(n), "alloc");
  k_tsdf_surface_emit<<<blocks_for(V.nvox, 256), 256, 0, st>>>(V.tsdf.p, V.weight.p, V.nx, V.ny, V.nz, flag.p,
                                                               slot.p, V.origin[0], V.origin[1], V.origin[2],
                                                               V.voxel, pos.p, nrm.p, conf.p, key.p);
  TCK(cudaGetLastError(), "emit");
  out->count = (int64_t)n;
  out->positions = (double*)std::malloc(3 * sizeof(double) * n);
  out->normals = (double*)std::malloc(3 * sizeof(double) * n);
  out->colors = (float*)std::calloc(3 * n, sizeof(float));
  out->confidences = (float*)std::malloc(sizeof(float) * n);
  out->keys = (int64_t*)std::malloc(sizeof(int64_t) * n);
  out->counts = (uint32_t*)std::malloc(sizeof(uint32_t) * n);
  if (!out->positions || !out->normals || !out->colors || !out->confidences || !out->keys || !out->counts) {
    recon_mvs_point_cloud_free(out);
    return tsdf_fail(RECON_ERR_OUT_OF_MEMORY, "tsdf_extract_points: host allocation failed");
  }
  for (size_t i = 0; i < n; ++i) out->counts[i] = 1u;
  cudaError_t e = cudaMemcpyAsync(out->positions, pos.p, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out->normals, nrm.p, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out->confidences, conf.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out->keys, key.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    recon_mvs_point_cloud_free(out);
    return cuda_fail(e, "extract download");
  }
  g_last_error.clear();
  return RECON_OK;
}

RECON_API recon_status recon_tsdf_dims(void* volume, int32_t* out_dims) {
  if (!volume || !out_dims) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_dims: NULL argument");
  const TsdfVolume& V = *static_cast<TsdfVolume*>(volume);
  out_dims[0] = V.nx;
  out_dims[1] = V.ny;
  out_dims[2] = V.nz;
  return RECON_OK;
}

RECON_API recon_status recon_tsdf_memory_usage(void* volume, uint64_t* out_bytes) {
  if (!volume || !out_bytes) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_memory_usage: NULL argument");
  const TsdfVolume& V = *static_cast<TsdfVolume*>(volume);
  *out_bytes = (uint64_t)V.nvox * 2 * sizeof(float);
  return RECON_OK;
}

RECON_API recon_status recon_tsdf_read_grid(void* volume, float* tsdf, float* weight) {
  if (!volume) return tsdf_fail(RECON_ERR_INVALID_ARGUMENT, "tsdf_read_grid: NULL volume");
  TsdfVolume& V = *static_cast<TsdfVolume*>(volume);
  TCK(cudaSetDevice(V.device), "set device");
  if (tsdf)
    TCK(cudaMemcpyAsync(tsdf, V.tsdf.p, V.nvox * sizeof(float), cudaMemcpyDeviceToHost, V.stream), "download");
  if (weight)
    TCK(cudaMemcpyAsync(weight, V.weight.p, V.nvox * sizeof(float), cudaMemcpyDeviceToHost, V.stream), "download");
  TCK(cudaStreamSynchronize(V.stream), "read grid");
  return RECON_OK;
}

RECON_API void recon_tsdf_destroy(void* volume) { delete static_cast<TsdfVolume*>(volume); }

}  // extern "C"
