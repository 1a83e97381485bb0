// noalloc.cu -- geometric consistency for callers that cannot allocate.
//
// Some callers must not have a library allocate device memory on their
// behalf: a capture or streaming loop that keeps every buffer in its own
// pre-sized pool (a cudaMalloc there would synchronise the whole device and
// stall the pipeline), or a host process that runs under a fixed GPU memory
// budget enforced by its own allocator.  Such callers already hold their
// depth maps and output masks in device memory.  For them,
// recon_mvs_geometric_consistency_noalloc runs the consistency kernel with
// the only device memory it needs beyond its inputs and outputs -- the
// per-source-map descriptor table -- placed in a fixed array that is part of
// this library's device image.  The entry point makes no cudaMalloc,
// cudaFree or other allocating call.
//
// The array holds at most kNoAllocMaxSources descriptors (64 source maps,
// about 9 KB); every GPU that loads the library keeps it until the process
// exits.  All calls share it, and it keeps the last call's contents: a call
// writes every descriptor it reads, so nothing in it has to start at zero.
// Calls whose work overlaps on the GPU (two streams, or two host threads)
// race on the array; serialise them.
#include <mutex>
#include <string>

#include "kernels.h"
#include "recon_mvs_gb300.h"

namespace rmvs {

constexpr int kNoAllocMaxSources = 64;

static __device__ __align__(256) ConsistencySrc g_noalloc_sources[kNoAllocMaxSources];
// Largest map side: keeps every pixel index inside a 32-bit int.
constexpr int kNoAllocMaxSide = 32768;

// the per-thread error text that recon_mvs_last_error() returns (engine.cu)
extern thread_local std::string g_last_error;

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the descriptor array on the current device, looked up
// once per device.  In host code g_noalloc_sources is only a host-side
// stand-in for the symbol, never a device address.
cudaError_t scratch_address(int device, ConsistencySrc** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sources);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[device] = p;
  }
  *out = static_cast<ConsistencySrc*>(g_noalloc_ptr[device]);
  return cudaSuccess;
}

// X_src = A X_ref + b with A = R_src R_ref^T, b = t_src - A t_ref, in the
// operation order the consistency kernel's bit-exact contract assumes.
void relative(const recon_pose& ref, const recon_pose& src, float Af[9], float bf[3]) {
  double A[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int q = 0; q < 3; ++q) s += src.r[i * 3 + q] * ref.r[j * 3 + q];
      A[i * 3 + j] = s;
    }
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += A[i * 3 + j] * ref.t[j];
    bf[i] = (float)(src.t[i] - s);
  }
  for (int i = 0; i < 9; ++i) Af[i] = (float)A[i];
}

}  // namespace
}  // namespace rmvs

using namespace rmvs;

extern "C" RECON_API recon_status recon_mvs_geometric_consistency_noalloc(
    const recon_mvs_depth_map* maps, const recon_pose* poses, const recon_camera_intrinsics* intr, int32_t num_maps,
    int32_t ref_index, float rel_depth_max, float reproj_px_max, int32_t min_views, uint8_t* out_count,
    uint8_t* out_keep, void* stream) {
  if (!maps || !poses || !intr || num_maps <= 0 || ref_index < 0 || ref_index >= num_maps || !out_count ||
      !out_keep || !maps[ref_index].depth || maps[ref_index].width <= 0 || maps[ref_index].height <= 0 ||
      maps[ref_index].width > kNoAllocMaxSide || maps[ref_index].height > kNoAllocMaxSide) {
    g_last_error = "geometric_consistency_noalloc: NULL pointer or bad map/index";
    return RECON_ERR_INVALID_ARGUMENT;
  }
  ConsistencySrc table[kNoAllocMaxSources];
  int n = 0;
  for (int s = 0; s < num_maps; ++s) {
    if (s == ref_index || !maps[s].depth || maps[s].width <= 0 || maps[s].height <= 0) continue;
    if (maps[s].width > kNoAllocMaxSide || maps[s].height > kNoAllocMaxSide) {
      g_last_error = "geometric_consistency_noalloc: a map larger than 32768 pixels on a side";
      return RECON_ERR_INVALID_ARGUMENT;
    }
    if (n == kNoAllocMaxSources) {
      g_last_error = "geometric_consistency_noalloc: more than 64 source maps (the fixed descriptor array's size)";
      return RECON_ERR_INVALID_ARGUMENT;
    }
    ConsistencySrc& c = table[n++];
    c.w = maps[s].width;
    c.h = maps[s].height;
    c.depth = maps[s].depth;
    c.fx = (float)intr[s].fx;
    c.fy = (float)intr[s].fy;
    c.cx = (float)intr[s].cx;
    c.cy = (float)intr[s].cy;
    relative(poses[ref_index], poses[s], c.A, c.b);
    relative(poses[s], poses[ref_index], c.Ai, c.bi);
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess || device < 0 || device >= kMaxDevices) {
    g_last_error = std::string("geometric_consistency_noalloc: no usable current device: ") + cudaGetErrorString(e);
    return RECON_ERR_MVS_GPU_FAILURE;
  }
  ConsistencySrc* dev_table = nullptr;
  e = scratch_address(device, &dev_table);
  if (e != cudaSuccess) {
    g_last_error = std::string("geometric_consistency_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return RECON_ERR_MVS_GPU_FAILURE;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n > 0) {
    // pageable source: the call returns once `table` has been read
    e = cudaMemcpyAsync(dev_table, table, sizeof(ConsistencySrc) * n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      g_last_error = std::string("geometric_consistency_noalloc: table upload: ") + cudaGetErrorString(e);
      return RECON_ERR_MVS_GPU_FAILURE;
    }
  }
  const recon_mvs_depth_map& R = maps[ref_index];
  ConsistencyRef ref{R.width, R.height, R.depth, (float)intr[ref_index].fx, (float)intr[ref_index].fy,
                     (float)intr[ref_index].cx, (float)intr[ref_index].cy};
  e = launch_consistency(ref, dev_table, n, rel_depth_max, reproj_px_max, min_views, out_count, out_keep, st);
  if (e != cudaSuccess) {
    g_last_error = std::string("geometric_consistency_noalloc: launch: ") + cudaGetErrorString(e);
    return RECON_ERR_MVS_GPU_FAILURE;
  }
  g_last_error.clear();
  return RECON_OK;
}
