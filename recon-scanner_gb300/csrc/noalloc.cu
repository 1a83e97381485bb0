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

// Device address of the descriptor array in the CURRENT context.  In host
// code g_noalloc_sources is only a host-side stand-in for the symbol, never a
// device address.  The address belongs to a CUDA context, not to a device
// number (a caller's own driver-API context, or a context re-created after
// cudaDeviceReset, maps the array elsewhere), so it is looked up on every
// call: the first call in a context loads the library's device image there
// (the set-up; it allocates the array as part of that image), and later
// calls are a table lookup that allocates nothing.
cudaError_t scratch_address(ConsistencySrc** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sources);
  if (e != cudaSuccess) return e;
  *out = static_cast<ConsistencySrc*>(p);
  return cudaSuccess;
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
    table[n++] = consistency_source(maps[s].width, maps[s].height, maps[s].depth, intr[s], poses[ref_index], poses[s]);
  }
  ConsistencySrc* dev_table = nullptr;
  cudaError_t e = scratch_address(&dev_table);
  if (e != cudaSuccess) {
    g_last_error = std::string("geometric_consistency_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return RECON_ERR_MVS_GPU_FAILURE;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n > 0) {
    // pageable source: the runtime copies `table` out before returning, which
    // may wait until the work already queued on the stream has drained
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
