// engine.cu -- host runtime of the GB300 MVS engine and its C ABI
// (include/recon_mvs_gb300.h).
//
// A Context owns one CUDA stream, reusable device workspaces and staged
// jobs (one reference view each: source textures, reference images, camera
// tables, search state).  Every entry point converts exceptions and CUDA
// errors into recon_status codes at the boundary (the reference's Guard,
// core/src/util/c_api.cpp:31-41); nothing here falls back to a CPU path.
//
// Host arithmetic that the bit-exact kernels depend on (relative transforms
// for the consistency test, baselines) is compiled with -ffp-contract=off.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cudaTypedefs.h>

#include "kernels.h"
#include "recon_mvs_gb300.h"

namespace rmvs {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
thread_local std::string g_last_error;

struct Failure : std::runtime_error {
  recon_status code;
  Failure(recon_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] static void fail(recon_status code, const std::string& msg) { throw Failure(code, msg); }

static void check_cuda(cudaError_t e, const char* what, const char* file, int line) {
  if (e == cudaSuccess) return;
  const std::string msg = std::string(what) + ": " + cudaGetErrorString(e) + " (" + file + ":" + std::to_string(line) + ")";
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(RECON_ERR_OUT_OF_MEMORY, msg);
  }
  fail(RECON_ERR_MVS_GPU_FAILURE, msg);
}
#define CK(x) check_cuda((x), #x, __FILE__, __LINE__)

template <class F>
static recon_status guard(F&& fn) {
  try {
    fn();
    g_last_error.clear();
    return RECON_OK;
  } catch (const Failure& f) {
    g_last_error = f.what();
    return f.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return RECON_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return RECON_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown exception";
    return RECON_ERR_INTERNAL;
  }
}

// ---------------------------------------------------------------------------
// device memory
// ---------------------------------------------------------------------------
template <class T>
struct DevArray {
  T* p = nullptr;
  size_t n = 0;
  DevArray() = default;
  DevArray(const DevArray&) = delete;
  DevArray& operator=(const DevArray&) = delete;
  ~DevArray() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count <= n && p) return;
    release();
    CK(cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T)));
    n = count;
  }
};

struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  void alloc(size_t b) {
    if (b <= bytes && p) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    CK(cudaMallocHost(&p, std::max<size_t>(b, 1)));
    bytes = b;
  }
};

struct Texture {
  cudaArray_t arr = nullptr;
  cudaTextureObject_t tex = 0;
  cudaTextureObject_t tex_lin = 0;
  ~Texture() {
    if (tex) cudaDestroyTextureObject(tex);
    if (tex_lin) cudaDestroyTextureObject(tex_lin);
    if (arr) cudaFreeArray(arr);
  }
};

// ---------------------------------------------------------------------------
// FP64 camera helpers in the reference's evaluation order
// ---------------------------------------------------------------------------
static void center_world(const recon_pose& p, double out[3]) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += p.r[j * 3 + i] * p.t[j];
    out[i] = -s;
  }
}

static double mean_baseline(const recon_pose& ref, const recon_pose* poses, const int32_t* idx, int n) {
  double rc[3];
  center_world(ref, rc);
  double sum = 0.0;
  for (int k = 0; k < n; ++k) {
    double sc[3], d[3];
    center_world(poses[idx[k]], sc);
    for (int i = 0; i < 3; ++i) d[i] = sc[i] - rc[i];
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s += d[i] * d[i];
    sum += std::sqrt(s);
  }
  return sum / (double)n;
}

// X_src = A X_ref + b with A = R_src R_ref^T, b = t_src - A t_ref
static ff ff_host(double d) {
  const float hi = (float)d;
  return ff{hi, (float)(d - (double)hi)};
}

static bool distorted(const recon_camera_intrinsics& k) {
  return k.k1 != 0.0 || k.k2 != 0.0 || k.k3 != 0.0 || k.p1 != 0.0 || k.p2 != 0.0;
}

static double depth_to_inverse_depth(double d) { return d < 1e-9 ? 1e9 : 1.0 / d; }

static int hardware_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return hw > 0 ? (int)hw : 1;
}

// ---------------------------------------------------------------------------
// jobs
// ---------------------------------------------------------------------------
// One staged image: its device copy (8-bit, or FP32 after on-device
// undistortion / pre-filtering) and, built on first use, its source form
// (a texture in the context's storage format) and its reference form
// ((I - 128) rows, the 2x2-box copy where needed, even / odd column planes).
// Jobs share images: a capture's view is staged once and serves as the
// reference of its own map and a source of the others.
struct StagedImage {
  int w = 0, h = 0;
  recon_camera_intrinsics intr{};  // as matched: distortion zeroed when undistorted on the device
  DevArray<uint8_t> u8;
  DevArray<float> f32;
  bool is_f32 = false;
  std::unique_ptr<Texture> tex;
  // the texel-pair image of `tex` and its TMA map (the staged-window
  // schedule's source), built on first use
  DevArray<float2> pair;
  DevArray<CUtensorMap> pair_map;
  DevArray<float> ref, box, de;
  int de_pitch = 0;  // floats per row of `de` (a multiple of 4: 16-byte rows for TMA)
  bool has_ref = false;
  std::shared_ptr<StagedImage> half;  // pyramid level 1, made on first use
  const void* dev() const { return is_f32 ? (const void*)f32.p : (const void*)u8.p; }
};

struct JobData {
  int w = 0, h = 0, num_src = 0;
  recon_mvs_config cfg{};
  recon_mvs_options opts{};
  bool degenerate = false;  // zero baseline or empty depth range: output all-invalid
  double inv_per_px = 0.0;
  std::shared_ptr<StagedImage> ref_img;
  std::vector<std::shared_ptr<StagedImage>> src_img;
  std::vector<SrcView> host_src;
  DevArray<SrcView> src_table;
  DevArray<float4> hyp;
  DevArray<float> cost;
  DevArray<uint8_t> support;
  DevArray<double> inv[2];
  DevArray<float> ccost[2];
  DevArray<int32_t> csup[2];
  std::vector<double> seeds;  // u, v, depth triples
  DevArray<float> seed_depth;
  int seed_gx = 0, seed_gy = 0;
  DevArray<float> out_depth, out_conf, out_normal, out_cost;
  DevArray<uint8_t> out_support;
  DevArray<unsigned int> filled;
  bool ran = false;
  Job J{};
  recon_pose ref_pose{};
  recon_camera_intrinsics ref_intr{};  // as matched (pinhole after undistortion)
  std::vector<recon_pose> src_pose;    // per relative source k
  std::unique_ptr<JobData> coarse;     // the half-resolution search of coarse-to-fine initialisation
};

// ---- plane-mode batch plans (used by the context below) ----
// Rows per sweep tile the autotuner chooses from (blocks of 32 x rows).
static const int kRowChoices[] = {2, 4, 8};
constexpr int kNumRowChoices = 3;
static int row_choice_index(int rows) {
  for (int i = 0; i < kNumRowChoices; ++i)
    if (kRowChoices[i] == rows) return i;
  return -1;
}

struct TuneKey {
  int device, patch_half, hw, storage, max_src, njobs;
  long long pixels;
  int staging;  // the schedules searched: 0 both, 1 texture reads only, 2 staged boxes only
  bool operator<(const TuneKey& o) const {
    return std::tie(device, patch_half, hw, storage, max_src, njobs, pixels, staging) <
           std::tie(o.device, o.patch_half, o.hw, o.storage, o.max_src, o.njobs, o.pixels, o.staging);
  }
};
struct TuneChoice {
  int rows = 4;
  int ctas_per_sm = 0;
  int staged = 0;
};
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneChoice>& tune_cache() {
  static std::map<TuneKey, TuneChoice> m;
  return m;
}

struct PlaneGroup {
  std::vector<JobData*> jobs;  // run order: iterations descending, then pixels descending
  int patch_half = 5;
  int mode = 0;  // source read mode (kSrcExact / kSrcTex / kSrcBf16)
  int max_src = 1, max_iters = 0;
  bool refine_any = false;  // some job refines by golden section
  bool refine_gn = false;   // some job refines by Gauss-Newton
  long long pixels = 0;
  std::unique_ptr<PlaneBatch> pix;                    // 32 x 4 pixel tiles
  std::unique_ptr<PlaneBatch> sweep[kNumRowChoices];  // 64-column x rows sweep tiles
  std::vector<int> active;  // active[it] = jobs with more than `it` iterations
  DevArray<int> queues;     // one work counter per half-sweep
  DevArray<CUtensorMap> tmaps[kNumRowChoices];  // per row choice, one per job (windows with H > 0)
  int rows = 4, ctas_per_sm = 1, grid = 1;
  bool can_stage = false;  // exact reads, 7x7 or 11x11, every source with a pair map
  int staged = 0;          // the sweep's window schedule: 1 = staged boxes

  int nj() const { return (int)jobs.size(); }
  const PlaneBatch& sweep_batch(int rows_) const { return *sweep[row_choice_index(rows_)]; }
  int sweep_total(int rows_, int it) const { return sweep_batch(rows_).start[active[it]]; }
};

struct PlanePlan {
  std::vector<int> ids;
  bool per_view = false;
  std::vector<std::unique_ptr<PlaneGroup>> groups;
  std::vector<std::unique_ptr<PlaneGroup>> coarse_groups;  // half-resolution searches, run in the init stage
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};  // init, sweeps, refine + output
  int sweep_launches = 0;
  ~PlanePlan() {
    for (auto e : exec)
      if (e) cudaGraphExecDestroy(e);
  }
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  recon_mvs_options opts{};
  std::map<int, std::unique_ptr<JobData>> jobs;
  int next_id = 1;
  std::unique_ptr<PlanePlan> plan;  // the last batch run, with its captured graph
  std::map<int, std::shared_ptr<StagedImage>> images;
  int next_image = 1;
  DevArray<unsigned long long> counter;
  DevArray<int> err;  // device-side failure flag (a TMA wait that ran out)
  bool test_tma_timeout = false;  // the next plane run injects a TMA wait that runs out
  DevArray<uint8_t> stage_u8;
  DevArray<float> stage_f32;
  DevArray<uint8_t> stage_tex;
  size_t stage_tex_pitch = 0;
  // compat draws (double-buffered)
  PinnedBuf draws_host[2], fire_host[2];
  DevArray<uint32_t> draws_dev[2];
  DevArray<uint8_t> fire_dev[2];
  cudaEvent_t copy_done[2] = {nullptr, nullptr};
  // device -> host downloads through two pinned chunks
  PinnedBuf d2h_buf[2];
  cudaEvent_t d2h_done[2] = {nullptr, nullptr};
  cudaEvent_t ev_start = nullptr, ev_sweep0 = nullptr, ev_sweep1 = nullptr, ev_end = nullptr;
  recon_mvs_stats stats{};

  explicit Context(const recon_mvs_options& o) : opts(o) {
    if (o.refine < 0 || o.refine > 2) fail(RECON_ERR_INVALID_ARGUMENT, "refine must be 0, 1 or 2");
    if (o.tile_rows != 0 && row_choice_index(o.tile_rows) < 0)
      fail(RECON_ERR_INVALID_ARGUMENT, "tile_rows must be 0 (autotuned), 2, 4 or 8");
    if (o.storage < RECON_MVS_STORAGE_FP32 || o.storage > RECON_MVS_STORAGE_U8)
      fail(RECON_ERR_INVALID_ARGUMENT, "unknown storage format");
    if (o.storage == RECON_MVS_STORAGE_U8 && o.mode != RECON_MVS_MODE_PLANE)
      fail(RECON_ERR_INVALID_ARGUMENT, "U8 storage needs plane mode");
    if (o.storage == RECON_MVS_STORAGE_BF16 && (o.mode != RECON_MVS_MODE_PLANE || o.interp != 0))
      fail(RECON_ERR_INVALID_ARGUMENT, "BF16 storage needs plane mode with exact interpolation (interp = 0)");
    if (o.exploration_iterations < 0) fail(RECON_ERR_INVALID_ARGUMENT, "exploration_iterations < 0");
    if (o.window_staging < 0 || o.window_staging > 2)
      fail(RECON_ERR_INVALID_ARGUMENT, "window_staging must be 0 (autotuned), 1 (off) or 2 (on)");
    if (o.window_staging == 2 &&
        (o.mode != RECON_MVS_MODE_PLANE || o.interp != 0 ||
         (o.storage != RECON_MVS_STORAGE_FP32 && o.storage != RECON_MVS_STORAGE_FP16)))
      fail(RECON_ERR_INVALID_ARGUMENT,
           "window_staging = 2 needs plane mode, exact interpolation and FP32 or FP16 storage");
    device = o.device;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (auto& e : copy_done) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : d2h_done) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(cudaEventCreate(&ev_start));
    CK(cudaEventCreate(&ev_sweep0));
    CK(cudaEventCreate(&ev_sweep1));
    CK(cudaEventCreate(&ev_end));
    counter.alloc(3);  // hypotheses, source windows sampled, of them read from staged boxes
    CK(cudaMemsetAsync(counter.p, 0, 3 * sizeof(unsigned long long), stream));
    err.alloc(1);
    CK(cudaMemsetAsync(err.p, 0, sizeof(int), stream));
  }
  ~Context() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    plan.reset();
    jobs.clear();
    images.clear();
    for (auto& e : copy_done)
      if (e) cudaEventDestroy(e);
    for (auto& e : d2h_done)
      if (e) cudaEventDestroy(e);
    for (auto e : {ev_start, ev_sweep0, ev_sweep1, ev_end})
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
  void use() const { CK(cudaSetDevice(device)); }
};

static void fill_defaults(recon_mvs_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->mode = RECON_MVS_MODE_PLANE;
  o->storage = RECON_MVS_STORAGE_FP32;
  o->best_k = 4;
  o->refine = 1;
  o->seed = 0x5DEECE66Dull;
  o->device = 0;
}

// Largest image side: the texture-gather limit of the device, which also
// keeps every pixel index (x + y * w) inside a 32-bit int.
constexpr int kMaxImageSide = 32768;

static void check_image_size(int w, int h, const char* what) {
  if (w <= 0 || h <= 0) fail(RECON_ERR_INVALID_ARGUMENT, std::string(what) + ": empty image");
  if (w > kMaxImageSide || h > kMaxImageSide)
    fail(RECON_ERR_INVALID_ARGUMENT, std::string(what) + ": image larger than 32768 pixels on a side");
}

// Pixels of a caller's depth map: 0 for a map without data or with a
// non-positive size (an empty map contributes nothing, as in the reference's
// loops); larger than the image limit is an error.
static size_t map_pixels(const recon_mvs_depth_map& m) {
  if (!m.depth || m.width <= 0 || m.height <= 0) return 0;
  check_image_size(m.width, m.height, "depth map");
  return (size_t)m.width * m.height;
}

// Contract checks of PatchMatchStereo (patchmatch_stereo.cpp:434-468).
static bool intrinsics_global(const recon_mvs_views& v) { return v.num_src_intrinsics == v.num_src_poses; }

static void validate_views(const recon_mvs_views* v) {
  if (!v) fail(RECON_ERR_INVALID_ARGUMENT, "views is NULL");
  if (!v->ref_gray || !v->ref_pose || !v->ref_intr) fail(RECON_ERR_INVALID_ARGUMENT, "reference image/pose/intrinsics NULL");
  check_image_size(v->ref_w, v->ref_h, "reference");
  if (v->num_src <= 0) fail(RECON_ERR_INVALID_ARGUMENT, "no source views");
  if (v->num_src > kMaxSources) fail(RECON_ERR_INVALID_ARGUMENT, "more than 32 source views");
  if (!v->src_gray || !v->src_w || !v->src_h || !v->src_poses || !v->src_intrinsics || !v->source_indices)
    fail(RECON_ERR_INVALID_ARGUMENT, "source arrays NULL");
  const bool glob = intrinsics_global(*v);
  const bool rel = v->num_src_intrinsics == v->num_src;
  if (!glob && !rel) fail(RECON_ERR_INVALID_ARGUMENT, "src_intrinsics length is neither the pose count nor the source count");
  for (int k = 0; k < v->num_src; ++k) {
    const int si = v->source_indices[k];
    if (si < 0 || si >= v->num_src_poses) fail(RECON_ERR_INVALID_ARGUMENT, "source index outside src_poses");
    if (!v->src_gray[k]) fail(RECON_ERR_INVALID_ARGUMENT, "source image NULL");
    check_image_size(v->src_w[k], v->src_h[k], "source");
  }
}

static const recon_camera_intrinsics& src_intr(const recon_mvs_views& v, int k) {
  return intrinsics_global(v) ? v.src_intrinsics[v.source_indices[k]] : v.src_intrinsics[k];
}

// Source texture of (I - 128) in the context's storage format: FP32, FP16
// (both with a point-filtered gather object and a linear-filter object),
// BF16 bits in a 16-bit unsigned channel (gather object only), or 8-bit
// unsigned read as normalised floats, I / 255 (both objects).
static void make_texture(Context& C, const void* dev_img_u8_or_f32, bool is_f32, int w, int h, int storage,
                         Texture& T) {
  const bool bf16 = storage == RECON_MVS_STORAGE_BF16;
  const bool u8 = storage == RECON_MVS_STORAGE_U8;
  cudaChannelFormatDesc desc = storage == RECON_MVS_STORAGE_FP16 ? cudaCreateChannelDescHalf()
                               : bf16 ? cudaCreateChannelDesc(16, 0, 0, 0, cudaChannelFormatKindUnsigned)
                               : u8   ? cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindUnsigned)
                                      : cudaCreateChannelDesc<float>();
  CK(cudaMallocArray(&T.arr, &desc, w, h, cudaArrayTextureGather));
  const size_t elem = storage == RECON_MVS_STORAGE_FP32 ? 4 : u8 ? 1 : 2;
  const size_t pitch = ((size_t)w * elem + 255) & ~(size_t)255;
  C.stage_tex.alloc(pitch * h);
  if (is_f32)
    CK(launch_prep_src_f32in((const float*)dev_img_u8_or_f32, w, h, C.stage_tex.p, pitch, storage, C.stream));
  else
    CK(launch_prep_src((const uint8_t*)dev_img_u8_or_f32, w, h, C.stage_tex.p, pitch, storage, C.stream));
  CK(cudaMemcpy2DToArrayAsync(T.arr, 0, 0, C.stage_tex.p, pitch, (size_t)w * elem, h, cudaMemcpyDeviceToDevice,
                              C.stream));
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof(rd));
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = T.arr;
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof(td));
  td.addressMode[0] = cudaAddressModeClamp;
  td.addressMode[1] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModePoint;
  td.readMode = u8 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
  td.normalizedCoords = 0;
  CK(cudaCreateTextureObject(&T.tex, &rd, &td, nullptr));
  if (!bf16) {
    td.filterMode = cudaFilterModeLinear;
    CK(cudaCreateTextureObject(&T.tex_lin, &rd, &td, nullptr));
  }
}

// Upload an 8-bit host image (optionally undistorted) to a device buffer;
// returns a device pointer to either u8 or f32 data (is_f32 set).
// An 8-bit image already on the device: undistortion (when `und` has
// distortion) and the optional pre-filter.  Returns the image to stage.
static const void* prepare_image(Context& C, int w, int h, const recon_camera_intrinsics* und, DevArray<uint8_t>& u8,
                                 DevArray<float>& f32, bool* is_f32);

static const void* upload_image(Context& C, const uint8_t* host, int w, int h, const recon_camera_intrinsics* und,
                                DevArray<uint8_t>& u8, DevArray<float>& f32, bool* is_f32) {
  u8.alloc((size_t)w * h);
  CK(cudaMemcpyAsync(u8.p, host, (size_t)w * h, cudaMemcpyHostToDevice, C.stream));
  return prepare_image(C, w, h, und, u8, f32, is_f32);
}

static const void* prepare_image(Context& C, int w, int h, const recon_camera_intrinsics* und, DevArray<uint8_t>& u8,
                                 DevArray<float>& f32, bool* is_f32) {
  const void* out = u8.p;
  *is_f32 = false;
  if (und && distorted(*und)) {
    f32.alloc((size_t)w * h);
    UndistortCam K{und->fx, und->fy, und->cx, und->cy, und->k1, und->k2, und->k3, und->p1, und->p2};
    CK(launch_undistort(u8.p, w, h, K, f32.p, C.stream));
    *is_f32 = true;
    out = f32.p;
  }
  if (C.opts.prefilter) {
    DevArray<float> tmp;
    tmp.alloc((size_t)w * h);
    CK(launch_binomial(*is_f32 ? nullptr : u8.p, *is_f32 ? f32.p : nullptr, w, h, tmp.p, C.stream));
    CK(cudaStreamSynchronize(C.stream));
    f32.alloc((size_t)w * h);
    CK(cudaMemcpyAsync(f32.p, tmp.p, (size_t)w * h * sizeof(float), cudaMemcpyDeviceToDevice, C.stream));
    CK(cudaStreamSynchronize(C.stream));
    *is_f32 = true;
    out = f32.p;
  }
  return out;
}

// Seeds -> per-32-px-cell mean depth (patchmatch_stereo.cpp:499-533).
static void cell_depths(const JobData& D, std::vector<double>* cell_sum, std::vector<int>* cell_n, int* gx, int* gy) {
  const int grid = 32;
  *gx = (D.w + grid - 1) / grid;
  *gy = (D.h + grid - 1) / grid;
  cell_sum->assign((size_t)(*gx) * (*gy), 0.0);
  cell_n->assign((size_t)(*gx) * (*gy), 0);
  for (size_t i = 0; i + 2 < D.seeds.size(); i += 3) {
    const double su = D.seeds[i], sv = D.seeds[i + 1], sd = D.seeds[i + 2];
    if (su < 0 || sv < 0 || su >= D.w || sv >= D.h) continue;
    if (sd <= 0.0) continue;
    const int cx = std::min(*gx - 1, (int)su / grid);
    const int cy = std::min(*gy - 1, (int)sv / grid);
    (*cell_sum)[(size_t)cy * (*gx) + cx] += sd;
    (*cell_n)[(size_t)cy * (*gx) + cx] += 1;
  }
}

// The reference -> source transform of one source (composed in FP64 in the
// reference's order) and the FP32 / float-float forms the kernels read.
static void set_src_transform(SrcView& S, const recon_pose& ref, const recon_pose& src,
                              const recon_camera_intrinsics& rk) {
  double A[9], b[3];
  relative_transform(ref, src, A, b);
  for (int i = 0; i < 9; ++i) {
    S.A[i] = A[i];
    S.Aff[i] = ff_host(A[i]);
  }
  for (int i = 0; i < 3; ++i) {
    S.bd[i] = b[i];
    S.b[i] = (float)b[i];
    S.bff[i] = ff_host(b[i]);
    S.Ac0[i] = (float)(A[i * 3 + 0] / rk.fx);
    S.Ac1[i] = (float)(A[i * 3 + 1] / rk.fy);
  }
}

static void zero_distortion(recon_camera_intrinsics* k) { k->k1 = k->k2 = k->k3 = k->p1 = k->p2 = 0.0; }

static std::shared_ptr<StagedImage> stage_image(Context& C, const uint8_t* host, int w, int h,
                                                const recon_camera_intrinsics& k, bool undistort) {
  if (!host) fail(RECON_ERR_INVALID_ARGUMENT, "image NULL");
  check_image_size(w, h, "staged");
  auto I = std::make_shared<StagedImage>();
  I->w = w;
  I->h = h;
  I->intr = k;
  upload_image(C, host, w, h, undistort ? &k : nullptr, I->u8, I->f32, &I->is_f32);
  if (undistort) zero_distortion(&I->intr);
  return I;
}

// A BGRA8 frame (rows `stride` bytes apart) converted to gray on the device
// with BgraToGray's integer weights (orchestrator.cpp:53-67), then staged as
// stage_image does.
static std::shared_ptr<StagedImage> stage_image_bgra(Context& C, const uint8_t* bgra, int w, int h, int stride,
                                                     const recon_camera_intrinsics& k, bool undistort) {
  check_image_size(w, h, "BGRA");
  if (!bgra || stride < 4 * w) fail(RECON_ERR_INVALID_ARGUMENT, "BGRA image NULL or short rows");
  auto I = std::make_shared<StagedImage>();
  I->w = w;
  I->h = h;
  I->intr = k;
  DevArray<uint8_t> dev;
  dev.alloc((size_t)4 * w * h);
  CK(cudaMemcpy2DAsync(dev.p, (size_t)4 * w, bgra, (size_t)stride, (size_t)4 * w, h, cudaMemcpyHostToDevice,
                       C.stream));
  I->u8.alloc((size_t)w * h);
  CK(launch_bgra_to_gray(dev.p, w, h, I->u8.p, C.stream));
  prepare_image(C, w, h, undistort ? &k : nullptr, I->u8, I->f32, &I->is_f32);
  CK(cudaStreamSynchronize(C.stream));  // the BGRA staging buffer is freed on return
  if (undistort) zero_distortion(&I->intr);
  return I;
}

static void ensure_texture(Context& C, StagedImage& I) {
  if (I.tex) return;
  I.tex = std::make_unique<Texture>();
  make_texture(C, I.dev(), I.is_f32, I.w, I.h, C.opts.storage, *I.tex);
  CK(cudaStreamSynchronize(C.stream));  // the context's staging buffer is reused
}

// cuTensorMapEncodeTiled through the runtime's driver entry point.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn) fail(RECON_ERR_MVS_GPU_FAILURE, "cuTensorMapEncodeTiled unavailable");
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  return encode;
}

// Sources get pair images when the staged-window schedule can apply: plane
// mode, exact interpolation, FP32 or FP16 storage, staging not switched off.
static bool wants_pairs(const Context& C) {
  return C.opts.mode == RECON_MVS_MODE_PLANE && C.opts.interp == 0 && C.opts.window_staging != 1 &&
         (C.opts.storage == RECON_MVS_STORAGE_FP32 || C.opts.storage == RECON_MVS_STORAGE_FP16);
}

// The texel-pair image of a staged image's texture -- {T(x, y), T(x + 1, y)}
// as two FP32 words, rows padded to an even count (16-byte pitch) -- and its
// 2-D TMA map of 8-byte elements, read in kStageW x kStageH boxes (zeros
// outside the image).
static void ensure_pair(Context& C, StagedImage& I) {
  if (I.pair_map.p) return;
  ensure_texture(C, I);
  const int pitch = (I.w + 1) & ~1;
  I.pair.alloc((size_t)pitch * I.h);
  CK(launch_pair_image(I.tex->tex, I.w, I.h, I.pair.p, pitch, C.stream));
  const cuuint64_t dims[2] = {(cuuint64_t)I.w, (cuuint64_t)I.h};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float2)};
  const cuuint32_t box[2] = {(cuuint32_t)kStageW, (cuuint32_t)kStageH};
  const cuuint32_t estr[2] = {1, 1};
  CUtensorMap map;
  const CUresult r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, I.pair.p, dims, strides, box, estr,
                                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(RECON_ERR_MVS_GPU_FAILURE, "cuTensorMapEncodeTiled failed (pair image)");
  I.pair_map.alloc(1);
  CK(cudaMemcpyAsync(I.pair_map.p, &map, sizeof(map), cudaMemcpyHostToDevice, C.stream));
  CK(cudaStreamSynchronize(C.stream));  // `map` lives on this stack frame
}

static void ensure_reference(Context& C, StagedImage& I) {
  if (I.has_ref) return;
  const bool plane = C.opts.mode == RECON_MVS_MODE_PLANE;
  const bool want_box = !plane || C.opts.sampling == 1;
  const size_t n = (size_t)I.w * I.h;
  I.ref.alloc(n);
  if (want_box) I.box.alloc(n);
  if (I.is_f32)
    CK(launch_prep_ref_f32(I.f32.p, I.w, I.h, I.ref.p, want_box ? I.box.p : nullptr, C.stream));
  else
    CK(launch_prep_ref(I.u8.p, I.w, I.h, I.ref.p, want_box ? I.box.p : nullptr, C.stream));
  if (plane) {
    const int half_w = (I.w + 1) / 2;
    I.de_pitch = (half_w + 3) & ~3;
    I.de.alloc((size_t)2 * I.de_pitch * I.h);
    CK(launch_deinterleave(C.opts.sampling == 1 ? I.box.p : I.ref.p, I.w, I.h, half_w, I.de_pitch, I.de.p,
                           C.stream));
  }
  I.has_ref = true;
}

// Pyramid level 1 of a staged image (kept with it: a capture's views are
// reduced once): 2 x 2 means, intrinsics of the half-resolution camera.
static std::shared_ptr<StagedImage> half_level(Context& C, const std::shared_ptr<StagedImage>& I) {
  if (I->half) return I->half;
  auto L = std::make_shared<StagedImage>();
  L->w = I->w / 2;
  L->h = I->h / 2;
  L->intr = I->intr;
  L->intr.fx *= 0.5;
  L->intr.fy *= 0.5;
  L->intr.cx *= 0.5;
  L->intr.cy *= 0.5;
  L->intr.width = L->w;
  L->intr.height = L->h;
  L->is_f32 = true;
  L->f32.alloc((size_t)L->w * L->h);
  CK(launch_half_level(I->is_f32 ? nullptr : I->u8.p, I->is_f32 ? I->f32.p : nullptr, I->w, I->h, L->f32.p,
                       C.stream));
  I->half = L;
  return L;
}

// Coarse-to-fine initialisation applies to a plane-mode job when it asks for
// fewer coarse iterations than its configuration runs and the half-resolution
// level still holds a few windows.
static int coarse_iterations(const Context& C, const recon_mvs_config& cfg, int w, int h) {
  const int n = C.opts.coarse_iterations;
  if (C.opts.mode != RECON_MVS_MODE_PLANE || n <= 0 || n >= cfg.iterations) return 0;
  const int min_side = 4 * (cfg.patch_size | 1);
  return (w / 2 >= min_side && h / 2 >= min_side) ? n : 0;
}

static std::unique_ptr<JobData> build_job_data(Context& C, const std::shared_ptr<StagedImage>& ref,
                                               const std::vector<std::shared_ptr<StagedImage>>& srcs,
                                               const recon_pose& ref_pose, const std::vector<recon_pose>& src_poses,
                                               const recon_mvs_config* cfg, const double* seeds, int num_seeds,
                                               bool coarse_level);

// A job from staged images: the reference, its sources and their poses.
static int build_job(Context& C, const std::shared_ptr<StagedImage>& ref,
                     const std::vector<std::shared_ptr<StagedImage>>& srcs, const recon_pose& ref_pose,
                     const std::vector<recon_pose>& src_poses, const recon_mvs_config* cfg, const double* seeds,
                     int num_seeds) {
  auto jd = build_job_data(C, ref, srcs, ref_pose, src_poses, cfg, seeds, num_seeds, false);
  const int id = C.next_id++;
  C.jobs[id] = std::move(jd);
  return id;
}

// `coarse_level`: the half-resolution search of another job (no seeds, no
// refinement, no outputs read).
static std::unique_ptr<JobData> build_job_data(Context& C, const std::shared_ptr<StagedImage>& ref,
                                               const std::vector<std::shared_ptr<StagedImage>>& srcs,
                                               const recon_pose& ref_pose, const std::vector<recon_pose>& src_poses,
                                               const recon_mvs_config* cfg, const double* seeds, int num_seeds,
                                               bool coarse_level) {
  if (!cfg) fail(RECON_ERR_INVALID_ARGUMENT, "config is NULL");
  if (cfg->patch_size < 1) fail(RECON_ERR_INVALID_ARGUMENT, "patch_size < 1");
  if (srcs.empty()) fail(RECON_ERR_INVALID_ARGUMENT, "no source views");
  if ((int)srcs.size() > kMaxSources) fail(RECON_ERR_INVALID_ARGUMENT, "more than 32 sources");
  C.use();
  auto jd = std::make_unique<JobData>();
  JobData& D = *jd;
  D.w = ref->w;
  D.h = ref->h;
  D.num_src = (int)srcs.size();
  D.cfg = *cfg;
  D.opts = C.opts;
  const bool plane = C.opts.mode == RECON_MVS_MODE_PLANE;
  const bool bf16 = C.opts.storage == RECON_MVS_STORAGE_BF16;
  const recon_camera_intrinsics rk = ref->intr;
  if (plane) {
    bool any = distorted(rk);
    for (const auto& I : srcs) any = any || distorted(I->intr);
    if (any) fail(RECON_ERR_INVALID_ARGUMENT, "plane mode needs pinhole images: stage with undistort = 1");
  }
  ensure_reference(C, *ref);
  D.ref_img = ref;
  const int half_w = (D.w + 1) / 2;

  // ---- sources ----
  D.host_src.resize(srcs.size());
  for (size_t k = 0; k < srcs.size(); ++k) {
    StagedImage& I = *srcs[k];
    ensure_texture(C, I);
    const recon_camera_intrinsics& sk = I.intr;
    SrcView& S = D.host_src[k];
    std::memset(&S, 0, sizeof(S));
    S.tex = I.tex->tex;
    S.tex_lin = I.tex->tex_lin;
    if (plane && wants_pairs(C) && (cfg->patch_size / 2 == 5 || cfg->patch_size / 2 == 3)) {
      ensure_pair(C, I);
      S.pair_map = I.pair_map.p;
    }
    S.w = I.w;
    S.h = I.h;
    S.fx = (float)sk.fx;
    S.fy = (float)sk.fy;
    S.cx = (float)sk.cx;
    S.cy = (float)sk.cy;
    S.ffx = ff_host(sk.fx);
    S.ffy = ff_host(sk.fy);
    S.fcx = ff_host(sk.cx);
    S.fcy = ff_host(sk.cy);
    S.k1 = (float)sk.k1;
    S.k2 = (float)sk.k2;
    S.k3 = (float)sk.k3;
    S.p1 = (float)sk.p1;
    S.p2 = (float)sk.p2;
    S.distorted = distorted(sk) ? 1 : 0;
    set_src_transform(S, ref_pose, src_poses[k], rk);
    D.src_pose.push_back(src_poses[k]);
  }
  D.src_img = srcs;
  D.ref_pose = ref_pose;
  D.ref_intr = rk;
  D.src_table.alloc(D.num_src);
  CK(cudaMemcpyAsync(D.src_table.p, D.host_src.data(), sizeof(SrcView) * D.num_src, cudaMemcpyHostToDevice,
                     C.stream));

  // ---- search range and baseline (patchmatch_stereo.cpp:473-485) ----
  std::vector<int32_t> ident(D.num_src);
  for (int k = 0; k < D.num_src; ++k) ident[k] = k;
  const double baseline = mean_baseline(ref_pose, src_poses.data(), ident.data(), D.num_src);
  const double inv_min = depth_to_inverse_depth(cfg->max_depth_m);
  const double inv_max = depth_to_inverse_depth(cfg->min_depth_m);
  D.degenerate = baseline < 1e-9 || !(inv_max > inv_min) || inv_min <= 0.0;
  const double focal_px = 0.5 * (rk.fx + rk.fy);
  D.inv_per_px = 1.0 / (focal_px * baseline);

  Job& J = D.J;
  std::memset(&J, 0, sizeof(J));
  J.w = D.w;
  J.h = D.h;
  J.num_src = D.num_src;
  J.patch_half = cfg->patch_size / 2;
  J.min_valid = cfg->patch_size * cfg->patch_size / 2;
  J.rfx = (float)rk.fx;
  J.rfy = (float)rk.fy;
  J.rcx = (float)rk.cx;
  J.rcy = (float)rk.cy;
  J.drfx = rk.fx;
  J.drfy = rk.fy;
  J.drcx = rk.cx;
  J.drcy = rk.cy;
  J.ffrx = ff_host(rk.fx);
  J.ffry = ff_host(rk.fy);
  J.ffrcx = ff_host(rk.cx);
  J.ffrcy = ff_host(rk.cy);
  J.ref_distorted = distorted(rk) ? 1 : 0;
  J.rk1 = rk.k1;
  J.rk2 = rk.k2;
  J.rk3 = rk.k3;
  J.rp1 = rk.p1;
  J.rp2 = rk.p2;
  J.ref = ref->ref.p;
  J.ref_box = ref->box.p;
  J.ref_de = ref->de.p;
  J.ref_half_w = half_w;
  J.ref_pitch = ref->de_pitch;
  J.half_pixel = (plane && C.opts.sampling == 1) ? 1 : 0;
  J.src_mode = !plane ? kSrcExact : (bf16 ? kSrcBf16 : (C.opts.interp == 1 ? kSrcTex : kSrcExact));
  J.pref = J.half_pixel ? ref->box.p : ref->ref.p;
  J.src = D.src_table.p;
  J.dinv_min = inv_min;
  J.dinv_max = inv_max;
  J.rho_min = (float)inv_min;
  J.rho_max = (float)inv_max;
  J.min_depth = cfg->min_depth_m;
  J.max_depth = cfg->max_depth_m;
  J.photo_threshold = (float)cfg->photo_threshold;
  J.best_k = C.opts.best_k;
  J.prune = C.opts.exhaustive ? 0 : 1;
  J.explore_iters = C.opts.exploration_iterations;
  J.seed = C.opts.seed;
  // the counters measure the full-resolution sweeps (the roofline's launches);
  // a coarse level's sweeps are not counted
  J.eval_counter = coarse_level ? nullptr : C.counter.p;

  const size_t npx = (size_t)D.w * D.h;
  if (plane) {
    D.hyp.alloc(npx);
    D.cost.alloc(npx);
    D.support.alloc(npx);
    J.hyp = D.hyp.p;
    J.cost = D.cost.p;
    J.support = D.support.p;
  } else {
    for (int i = 0; i < 2; ++i) {
      D.inv[i].alloc(npx);
      D.ccost[i].alloc(npx);
      D.csup[i].alloc(npx);
    }
    J.inv = D.inv[0].p;
    J.isupport = D.csup[0].p;
  }
  if (seeds && num_seeds > 0) D.seeds.assign(seeds, seeds + 3 * (size_t)num_seeds);
  D.out_depth.alloc(npx);
  D.out_conf.alloc(npx);
  D.out_support.alloc(npx);
  if (plane) {
    D.out_normal.alloc(npx * 3);
  }
  D.out_cost.alloc(npx);
  D.filled.alloc(1);
  if (plane) {
    if (!D.seeds.empty()) {
      // seeds -> per-32-px-cell mean depth (patchmatch_stereo.cpp:499-533)
      std::vector<double> sum;
      std::vector<int> cnt;
      int gx, gy;
      cell_depths(D, &sum, &cnt, &gx, &gy);
      std::vector<float> sd(sum.size(), 0.f);
      for (size_t i = 0; i < sum.size(); ++i)
        if (cnt[i] > 0) sd[i] = (float)(sum[i] / (double)cnt[i]);
      D.seed_depth.alloc(sd.size());
      CK(cudaMemcpyAsync(D.seed_depth.p, sd.data(), sd.size() * sizeof(float), cudaMemcpyHostToDevice, C.stream));
      D.seed_gx = gx;
      J.seed_depth = D.seed_depth.p;
      J.seed_gx = gx;
    }
    J.iterations = cfg->iterations;
    // golden section: subpixel_iterations steps (the reference's schedule);
    // Gauss-Newton: one Levenberg-Marquardt step (up to four damping
    // retries) -- further steps did not lower the error at the measured
    // image noise, and each costs about one golden-section search
    J.refine_iters = (C.opts.refine && cfg->subpixel_iterations > 0 && !coarse_level)
                         ? (C.opts.refine == 2 ? 1 : cfg->subpixel_iterations)
                         : 0;
    J.refine_mode = C.opts.refine;
    J.inv_per_px = (float)D.inv_per_px;
    J.out_depth = D.out_depth.p;
    J.out_support = D.out_support.p;
    J.out_conf = D.out_conf.p;
    J.out_normal = D.out_normal.p;
    J.out_cost = D.out_cost.p;
    J.out_filled = D.filled.p;
    const int nc = coarse_level ? 0 : coarse_iterations(C, *cfg, D.w, D.h);
    if (nc > 0) {
      std::vector<std::shared_ptr<StagedImage>> half_srcs;
      for (const auto& I : srcs) half_srcs.push_back(half_level(C, I));
      recon_mvs_config c1 = *cfg;
      c1.iterations = nc;
      D.coarse = build_job_data(C, half_level(C, ref), half_srcs, ref_pose, src_poses, &c1, nullptr, 0, true);
      const JobData& L = *D.coarse;
      J.coarse_hyp = L.hyp.p;
      J.coarse_cost = L.cost.p;
      J.coarse_w = L.w;
      J.coarse_h = L.h;
      J.crfx = L.J.rfx;
      J.crfy = L.J.rfy;
      J.crcx = L.J.rcx;
      J.crcy = L.J.rcy;
      J.iter_offset = nc;
      J.iterations = cfg->iterations - nc;
    }
  }
  CK(cudaStreamSynchronize(C.stream));
  return jd;
}

// The PatchMatchStereo argument list (reference index contract): every image
// staged for this job alone.
static int stage_job(Context& C, const recon_mvs_views* v, const recon_mvs_config* cfg, bool undistort,
                     const double* seeds, int num_seeds) {
  validate_views(v);
  if (!cfg) fail(RECON_ERR_INVALID_ARGUMENT, "config is NULL");
  C.use();
  const bool plane = C.opts.mode == RECON_MVS_MODE_PLANE;
  if (plane && !undistort) {
    bool any = distorted(*v->ref_intr);
    for (int k = 0; k < v->num_src; ++k) any = any || distorted(src_intr(*v, k));
    if (any) fail(RECON_ERR_INVALID_ARGUMENT, "plane mode needs pinhole images: stage with undistort = 1");
  }
  auto ref = stage_image(C, v->ref_gray, v->ref_w, v->ref_h, *v->ref_intr, undistort);
  std::vector<std::shared_ptr<StagedImage>> srcs;
  std::vector<recon_pose> poses;
  for (int k = 0; k < v->num_src; ++k) {
    srcs.push_back(stage_image(C, v->src_gray[k], v->src_w[k], v->src_h[k], src_intr(*v, k), undistort));
    poses.push_back(v->src_poses[v->source_indices[k]]);
  }
  return build_job(C, ref, srcs, *v->ref_pose, poses, cfg, seeds, num_seeds);
}

static JobData& get_job(Context& C, int id) {
  auto it = C.jobs.find(id);
  if (it == C.jobs.end()) fail(RECON_ERR_INVALID_ARGUMENT, "unknown job id");
  return *it->second;
}

// ---- plane mode -----------------------------------------------------------
// Plane-mode jobs run in batches: the jobs of one recon_mvs_jobs_run call that
// share the window size and interpolation mode form a group, and each stage
// (init, every half-sweep, refinement, output) is ONE launch over the whole
// group -- the half-sweeps a persistent kernel pulling tiles of all the
// group's views from a work counter.  The run is captured once as a CUDA
// graph and replayed while the same jobs are run again.  The per-view form
// (options.per_view = 1) launches the same kernels once per view instead,
// without a graph: the comparison the batched form is measured against.

// The TMA view of a job's reference planes: a 3-D tensor {half_w, h, 2} of
// FP32 with 16-byte row pitch, read in boxes of kTileCols columns x box_rows
// rows x both planes (what one sweep tile stages), zeros outside.
static void encode_ref_tile_map(const JobData& D, int box_rows, CUtensorMap* out) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  const Job& J = D.J;
  const cuuint64_t dims[3] = {(cuuint64_t)J.ref_half_w, (cuuint64_t)J.h, 2};
  const cuuint64_t strides[2] = {(cuuint64_t)J.ref_pitch * sizeof(float),
                                 (cuuint64_t)J.ref_pitch * sizeof(float) * (cuuint64_t)J.h};
  const cuuint32_t box[3] = {(cuuint32_t)kTileCols, (cuuint32_t)box_rows, 2};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(J.ref_de), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(RECON_ERR_MVS_GPU_FAILURE, "cuTensorMapEncodeTiled failed");
}

static void build_group(Context& C, PlaneGroup& G) {
  std::stable_sort(G.jobs.begin(), G.jobs.end(), [](const JobData* a, const JobData* b) {
    if (a->J.iterations != b->J.iterations) return a->J.iterations > b->J.iterations;
    return (long long)a->w * a->h > (long long)b->w * b->h;
  });
  const int n = G.nj();
  if (n < 1 || n > kBatchJobs) fail(RECON_ERR_INTERNAL, "batch group size out of range");
  G.pix = std::make_unique<PlaneBatch>();
  std::memset(G.pix.get(), 0, sizeof(PlaneBatch));
  for (auto& b : G.sweep) {
    b = std::make_unique<PlaneBatch>();
    std::memset(b.get(), 0, sizeof(PlaneBatch));
  }
  G.max_src = 1;
  G.max_iters = 0;
  G.refine_any = false;
  G.refine_gn = false;
  G.pixels = 0;
  for (int j = 0; j < n; ++j) {
    const JobData& D = *G.jobs[j];
    G.max_src = std::max(G.max_src, D.num_src);
    G.max_iters = std::max(G.max_iters, std::max(0, D.J.iterations));
    G.refine_any = G.refine_any || (D.J.refine_iters > 0 && D.J.refine_mode == 1);
    G.refine_gn = G.refine_gn || (D.J.refine_iters > 0 && D.J.refine_mode == 2);
    G.pixels += (long long)D.w * D.h;
    auto add = [&](PlaneBatch& B, long long tiles) {
      B.jobs[j] = D.J;
      const long long next = (long long)B.start[j] + tiles;
      if (next > 0x7fffffffLL) fail(RECON_ERR_INVALID_ARGUMENT, "batch too large: more than 2^31 tiles");
      B.start[j + 1] = (int)next;
      B.njobs = n;
    };
    add(*G.pix, (long long)((D.w + 31) / 32) * ((D.h + 3) / 4));
    for (int r = 0; r < kNumRowChoices; ++r)
      add(*G.sweep[r], (long long)((D.w + 63) / 64) * ((D.h + kRowChoices[r] - 1) / kRowChoices[r]));
  }
  G.pix->err = C.err.p;
  for (int r = 0; r < kNumRowChoices; ++r) {
    G.sweep[r]->err = C.err.p;
    G.sweep[r]->tma_skip = C.test_tma_timeout ? 1 : 0;
    G.sweep[r]->tma_poll_limit = C.test_tma_timeout ? 4096 : 0;
    if (G.patch_half != 5 && G.patch_half != 3) continue;  // the generic window reads global memory
    std::vector<CUtensorMap> maps(n);
    for (int j = 0; j < n; ++j) encode_ref_tile_map(*G.jobs[j], kRowChoices[r] + 2 * G.patch_half, &maps[j]);
    G.tmaps[r].alloc(n);
    CK(cudaMemcpy(G.tmaps[r].p, maps.data(), sizeof(CUtensorMap) * n, cudaMemcpyHostToDevice));
    G.sweep[r]->tmaps = G.tmaps[r].p;
  }
  G.can_stage = G.mode == kSrcExact && (G.patch_half == 5 || G.patch_half == 3);
  for (int j = 0; j < n && G.can_stage; ++j)
    for (const SrcView& S : G.jobs[j]->host_src) G.can_stage = G.can_stage && S.pair_map != nullptr;
  G.active.assign(std::max(G.max_iters, 1), 0);
  for (int it = 0; it < G.max_iters; ++it)
    for (int j = 0; j < n; ++j)
      if (G.jobs[j]->J.iterations > it) G.active[it] = j + 1;
  G.queues.alloc(std::max(2 * G.max_iters, 1));
}

static int sm_count(int device) {
  int n = 0;
  CK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device));
  return std::max(n, 1);
}

// The autotuner: times one half-sweep of the group itself for every window
// schedule (texture reads, or staged boxes where exact reads allow them),
// tile shape (rows per tile) and persistent grid (resident blocks per SM,
// full or one less), starting each trial from a fresh init, and keeps the
// fastest.  The choice cannot change results -- every pixel computes the same
// thing whatever the tile or schedule -- and is cached per (device, window,
// interpolation, storage, max sources, job count, pixel count, staging
// option).  Explicit options.tile_rows skips the search (and takes staged
// boxes only when window_staging = 2).
static void tune_group(Context& C, PlaneGroup& G) {
  const int nsm = sm_count(C.device);
  auto set_shape = [&](int rows, int ctas, int staged) {
    G.rows = rows;
    G.ctas_per_sm = ctas;
    G.grid = ctas * nsm;
    G.staged = staged;
  };
  auto occupancy = [&](int rows, int staged) {
    int b = 0;
    CK(plane_sweep_occupancy(G.patch_half, G.mode, G.max_src, rows, staged, &b));
    return b;
  };
  // the window schedules to consider: staged boxes only where they apply
  const int stage_lo = (G.can_stage && C.opts.window_staging == 2) ? 1 : 0;
  const int stage_hi = (G.can_stage && C.opts.window_staging != 1) ? 1 : 0;
  if (C.opts.tile_rows != 0) {
    const int b = occupancy(C.opts.tile_rows, stage_lo);
    if (b < 1) fail(RECON_ERR_INVALID_ARGUMENT, "tile_rows: the sweep kernel does not fit on an SM");
    set_shape(C.opts.tile_rows, b, stage_lo);
    return;
  }
  const TuneKey key{C.device, G.patch_half, G.mode, C.opts.storage, G.max_src, G.nj(), G.pixels,
                    C.opts.window_staging};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = tune_cache().find(key);
    if (it != tune_cache().end()) {
      set_shape(it->second.rows, it->second.ctas_per_sm, it->second.staged);
      return;
    }
  }
  if (G.max_iters == 0) {
    set_shape(4, std::max(1, occupancy(4, stage_lo)), stage_lo);
    return;
  }
  unsigned long long saved[3] = {0, 0, 0};
  CK(cudaMemcpyAsync(saved, C.counter.p, sizeof(saved), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaStreamSynchronize(C.stream));
  float best_ms = 1e30f;
  TuneChoice best;
  best.staged = stage_lo;
  for (int staged = stage_lo; staged <= stage_hi; ++staged)
    for (int rows : kRowChoices) {
      const int b = occupancy(rows, staged);
      for (int ctas = b; ctas >= std::max(1, b - 1); --ctas) {
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {  // the first trial also loads the kernel
          CK(launch_plane_init(*G.pix, G.patch_half, G.mode, G.max_src, G.queues.p, (int)G.queues.n, C.stream));
          CK(cudaEventRecord(C.ev_sweep0, C.stream));
          CK(launch_plane_sweep(G.sweep_batch(rows), G.sweep_total(rows, 0), G.queues.p, G.patch_half, G.mode,
                                G.max_src, rows, staged, ctas * nsm, 0, 0, C.stream));
          CK(cudaEventRecord(C.ev_sweep1, C.stream));
          CK(cudaEventSynchronize(C.ev_sweep1));
          CK(cudaEventElapsedTime(&ms, C.ev_sweep0, C.ev_sweep1));
        }
        if (ms < best_ms) {
          best_ms = ms;
          best.rows = rows;
          best.ctas_per_sm = ctas;
          best.staged = staged;
        }
      }
    }
  if (best_ms >= 1e30f) fail(RECON_ERR_MVS_GPU_FAILURE, "the sweep kernel does not fit on an SM");
  CK(cudaMemcpyAsync(C.counter.p, saved, sizeof(saved), cudaMemcpyHostToDevice, C.stream));
  CK(cudaStreamSynchronize(C.stream));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache()[key] = best;
  }
  set_shape(best.rows, best.ctas_per_sm, best.staged);
  C.stats.tune_trials += 1;
}

// The run of a plan in three stages -- every group's init; the sweeps;
// every group's refinement and output -- each captured as its own CUDA graph
// in the batched form, so that the context's timing events sit on the stream
// between the graph launches and bracket the sweeps exactly.
static void enqueue_stage(Context& C, PlanePlan& P, int stage) {
  if (stage == 0) {
    // coarse-to-fine: the half-resolution searches first; the full-resolution
    // init then starts each pixel from its parent's plane
    for (auto& g : P.coarse_groups) {
      PlaneGroup& G = *g;
      CK(launch_plane_init(*G.pix, G.patch_half, G.mode, G.max_src, G.queues.p, (int)G.queues.n, C.stream));
      for (int it = 0; it < G.max_iters; ++it)
        for (int color = 0; color < 2; ++color)
          CK(launch_plane_sweep(G.sweep_batch(G.rows), G.sweep_total(G.rows, it), G.queues.p + 2 * it + color,
                                G.patch_half, G.mode, G.max_src, G.rows, G.staged, G.grid, color, it, C.stream));
    }
    for (auto& g : P.groups) {
      PlaneGroup& G = *g;
      CK(launch_plane_init(*G.pix, G.patch_half, G.mode, G.max_src, G.queues.p, (int)G.queues.n, C.stream));
    }
  } else if (stage == 1) {
    int launches = 0;
    for (auto& g : P.groups) {
      PlaneGroup& G = *g;
      for (int it = 0; it < G.max_iters; ++it)
        for (int color = 0; color < 2; ++color) {
          CK(launch_plane_sweep(G.sweep_batch(G.rows), G.sweep_total(G.rows, it), G.queues.p + 2 * it + color,
                                G.patch_half, G.mode, G.max_src, G.rows, G.staged, G.grid, color, it, C.stream));
          ++launches;
        }
    }
    P.sweep_launches = launches;
  } else {
    for (auto& g : P.groups) {
      PlaneGroup& G = *g;
      if (G.refine_any) CK(launch_plane_refine(*G.pix, G.patch_half, G.mode, G.max_src, C.stream));
      if (G.refine_gn) CK(launch_plane_refine_gn(*G.pix, G.patch_half, G.mode, G.max_src, C.stream));
      CK(launch_plane_output(*G.pix, C.stream));
    }
  }
}

static void capture_stage(Context& C, PlanePlan& P, int stage) {
  CK(cudaStreamBeginCapture(C.stream, cudaStreamCaptureModeThreadLocal));
  cudaGraph_t graph = nullptr;
  try {
    enqueue_stage(C, P, stage);
  } catch (...) {
    cudaStreamEndCapture(C.stream, &graph);
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    throw;
  }
  CK(cudaStreamEndCapture(C.stream, &graph));
  const cudaError_t e = cudaGraphInstantiate(&P.exec[stage], graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
}

static void launch_plan(Context& C, PlanePlan& P) {
  const cudaEvent_t marks[4] = {C.ev_start, C.ev_sweep0, C.ev_sweep1, C.ev_end};
  CK(cudaEventRecord(marks[0], C.stream));
  for (int stage = 0; stage < 3; ++stage) {
    if (P.exec[stage])
      CK(cudaGraphLaunch(P.exec[stage], C.stream));
    else
      enqueue_stage(C, P, stage);
    CK(cudaEventRecord(marks[stage + 1], C.stream));
  }
}

static std::unique_ptr<PlanePlan> make_plan(Context& C, const std::vector<JobData*>& jobs,
                                            const std::vector<int>& ids) {
  auto P = std::make_unique<PlanePlan>();
  P->ids = ids;
  P->per_view = C.opts.per_view != 0;
  auto group = [&](const std::vector<JobData*>& list, std::vector<std::unique_ptr<PlaneGroup>>& groups) {
    for (JobData* D : list) {
      PlaneGroup* G = nullptr;
      if (!P->per_view)
        for (auto& g : groups)
          if (g->patch_half == D->J.patch_half && g->mode == D->J.src_mode && g->nj() < kBatchJobs) G = g.get();
      if (!G) {
        groups.push_back(std::make_unique<PlaneGroup>());
        G = groups.back().get();
        G->patch_half = D->J.patch_half;
        G->mode = D->J.src_mode;
      }
      G->jobs.push_back(D);
    }
    for (auto& g : groups) build_group(C, *g);
    for (auto& g : groups) tune_group(C, *g);
  };
  std::vector<JobData*> coarse;
  for (JobData* D : jobs)
    if (D->coarse) coarse.push_back(D->coarse.get());
  group(coarse, P->coarse_groups);
  group(jobs, P->groups);
  if (!P->per_view)
    for (int stage = 0; stage < 3; ++stage) capture_stage(C, *P, stage);
  else
    P->sweep_launches = 0;
  return P;
}

static void run_plane_jobs(Context& C, const std::vector<JobData*>& jobs, const std::vector<int>& ids) {
  if (jobs.empty()) return;
  if (!C.plan || C.plan->ids != ids || C.plan->per_view != (C.opts.per_view != 0) || C.test_tma_timeout) {
    C.plan.reset();
    C.plan = make_plan(C, jobs, ids);
  }
  PlanePlan& P = *C.plan;
  launch_plan(C, P);
  if (C.test_tma_timeout) {
    // the injection lasts one run: the next run rebuilds its plan
    CK(cudaStreamSynchronize(C.stream));
    C.test_tma_timeout = false;
    C.plan.reset();
    C.stats.last_sweep_launches = 0;
    return;
  }
  if (P.exec[0]) C.stats.graph_launches += 1;
  C.stats.last_sweep_launches = P.sweep_launches;
  C.stats.tile_rows = P.groups[0]->rows;
  C.stats.ctas_per_sm = P.groups[0]->ctas_per_sm;
  C.stats.window_staging = P.groups[0]->staged;
}

// ---- compat mode ----------------------------------------------------------
// The reference's random init (one global xorshift in row-major order after
// seeding, :487-539) and its per-sweep row-block draws (:612-660).
struct XorShift {
  uint64_t s;
  explicit XorShift(uint64_t seed) : s(seed ? seed : 0x9E3779B97F4A7C15ull) {}
  uint32_t next() {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return (uint32_t)((s * 0x2545F4914F6CDD1Dull) >> 32);
  }
};

static int resolve_threads(const recon_mvs_config& c) {
  int t = c.num_threads;
  if (t <= 0) t = hardware_threads();
  return std::max(1, t);
}

static void gen_draws(const JobData& D, int iter, int dir, uint32_t* draws, uint8_t* fire) {
  const int W = D.w, H = D.h;
  const int count = D.cfg.random_search_count > 0 ? D.cfg.random_search_count : 0;
  const int stride = count + 1;
  const int threads = resolve_threads(D.cfg);
  const int block_count = std::min(threads, std::max(1, H / 16));
  const int rows_per_block = (H + block_count - 1) / block_count;
  const bool reverse_x = (dir == 1 || dir == 3);
  const bool reverse_y = (dir >= 2);
  const double restart = D.cfg.restart_ratio;
  auto one = [&](int b) {
    const int yb0 = b * rows_per_block;
    const int yb1 = std::min(H, yb0 + rows_per_block);
    if (yb0 >= yb1) return;
    XorShift rng(0x5DEECE66Dull + (uint64_t)b * 0x9E3779B97F4A7C15ull + (uint64_t)iter * 0xC2B2AE3D27D4EB4Full);
    const int y_start = reverse_y ? yb1 - 1 : yb0, y_end = reverse_y ? yb0 - 1 : yb1, y_step = reverse_y ? -1 : 1;
    for (int y = y_start; y != y_end; y += y_step) {
      const int x_start = reverse_x ? W - 1 : 0, x_end = reverse_x ? -1 : W, x_step = reverse_x ? -1 : 1;
      for (int x = x_start; x != x_end; x += x_step) {
        const size_t idx = (size_t)y * W + x;
        uint32_t* d = draws + idx * stride;
        for (int k = 0; k < count; ++k) d[k] = rng.next();
        const uint32_t t = rng.next();
        const bool f = ((double)t / 4294967296.0) < restart;
        fire[idx] = f ? 1 : 0;
        d[count] = f ? rng.next() : 0u;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int b = 1; b < block_count; ++b) pool.emplace_back(one, b);
  one(0);
  for (auto& t : pool) t.join();
}

static void run_compat(Context& C, JobData& D) {
  Job& J = D.J;
  const size_t npx = (size_t)D.w * D.h;
  // initial inverse depths (host, the reference's generator)
  std::vector<double> inv(npx, 0.0);
  std::vector<uint8_t> init(npx, 0);
  if (!D.seeds.empty()) {
    std::vector<double> sum;
    std::vector<int> cnt;
    int gx, gy;
    cell_depths(D, &sum, &cnt, &gx, &gy);
    for (int y = 0; y < D.h; ++y)
      for (int x = 0; x < D.w; ++x) {
        const int cx = std::min(gx - 1, x / 32), cy = std::min(gy - 1, y / 32);
        const size_t c = (size_t)cy * gx + cx;
        if (cnt[c] == 0) continue;
        inv[(size_t)y * D.w + x] = depth_to_inverse_depth(sum[c] / (double)cnt[c]);
        init[(size_t)y * D.w + x] = 1;
      }
  }
  XorShift rng(0x5DEECE66Dull);
  for (size_t i = 0; i < npx; ++i) {
    if (init[i]) continue;
    inv[i] = J.dinv_min + ((double)rng.next() / 4294967296.0) * (J.dinv_max - J.dinv_min);
  }
  CK(cudaEventRecord(C.ev_start, C.stream));
  CK(cudaMemcpyAsync(D.inv[0].p, inv.data(), npx * sizeof(double), cudaMemcpyHostToDevice, C.stream));
  J.inv = D.inv[0].p;
  J.isupport = D.csup[0].p;
  CK(launch_compat_init(J, D.ccost[0].p, C.stream));
  CK(cudaEventRecord(C.ev_sweep0, C.stream));
  const int count = std::max(0, D.cfg.random_search_count);
  const int stride = count + 1;
  const int dirs = std::max(1, D.cfg.propagation_directions);
  int cur = 0, sweep = 0;
  for (int it = 0; it < D.cfg.iterations; ++it)
    for (int dir = 0; dir < dirs; ++dir, ++sweep) {
      const int j = sweep & 1;
      if (sweep >= 2) CK(cudaEventSynchronize(C.copy_done[j]));
      C.draws_host[j].alloc(npx * stride * sizeof(uint32_t));
      C.fire_host[j].alloc(npx);
      gen_draws(D, it, dir, (uint32_t*)C.draws_host[j].p, (uint8_t*)C.fire_host[j].p);
      C.draws_dev[j].alloc(npx * stride);
      C.fire_dev[j].alloc(npx);
      CK(cudaMemcpyAsync(C.draws_dev[j].p, C.draws_host[j].p, npx * stride * sizeof(uint32_t), cudaMemcpyHostToDevice,
                         C.stream));
      CK(cudaMemcpyAsync(C.fire_dev[j].p, C.fire_host[j].p, npx, cudaMemcpyHostToDevice, C.stream));
      CK(cudaEventRecord(C.copy_done[j], C.stream));
      const int nxt = cur ^ 1;
      CK(launch_compat_sweep(J, D.inv[cur].p, D.ccost[cur].p, D.csup[cur].p, D.inv[nxt].p, D.ccost[nxt].p,
                             D.csup[nxt].p, C.draws_dev[j].p, C.fire_dev[j].p, stride, count,
                             D.cfg.random_search_radius_ratio, D.cfg.propagation_enabled, C.stream));
      cur = nxt;
    }
  CK(cudaEventRecord(C.ev_sweep1, C.stream));
  CK(cudaMemsetAsync(D.filled.p, 0, sizeof(unsigned int), C.stream));
  CK(launch_compat_output(J, D.inv[cur].p, D.ccost[cur].p, D.csup[cur].p, D.out_depth.p, D.out_support.p,
                          D.out_conf.p, D.filled.p, C.stream));
  CK(cudaMemcpyAsync(D.out_cost.p, D.ccost[cur].p, npx * sizeof(float), cudaMemcpyDeviceToDevice, C.stream));
  CK(cudaEventRecord(C.ev_end, C.stream));
  C.stats.last_sweep_launches = sweep;
}

// Runs jobs in the given order: plane-mode jobs as one batch, compat-mode
// jobs (the reference's own sweep order) one after another.
static void run_jobs(Context& C, const std::vector<int>& ids) {
  C.use();
  std::vector<JobData*> plane;
  std::vector<int> plane_ids;
  for (int id : ids) {
    JobData& D = get_job(C, id);
    if (D.degenerate) continue;
    if (D.opts.mode == RECON_MVS_MODE_PLANE) {
      if (std::find(plane_ids.begin(), plane_ids.end(), id) != plane_ids.end())
        fail(RECON_ERR_INVALID_ARGUMENT, "a job is listed twice");
      plane.push_back(&D);
      plane_ids.push_back(id);
    } else {
      run_compat(C, D);
    }
  }
  run_plane_jobs(C, plane, plane_ids);
  for (int id : ids) get_job(C, id).ran = true;
}

static void run_job(Context& C, int id) { run_jobs(C, std::vector<int>{id}); }

// Drops a job, and the cached plan when it runs that job.
static void erase_job(Context& C, int id) {
  if (C.plan && std::find(C.plan->ids.begin(), C.plan->ids.end(), id) != C.plan->ids.end()) {
    cudaStreamSynchronize(C.stream);
    C.plan.reset();
  }
  C.jobs.erase(id);
}

// A device-side failure (a TMA wait that ran out) becomes MVS_GPU_FAILURE;
// the flag is cleared so the context stays usable.
static void check_device_error(Context& C) {
  int e = 0;
  CK(cudaMemcpy(&e, C.err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    CK(cudaMemset(C.err.p, 0, sizeof(int)));
    fail(RECON_ERR_MVS_GPU_FAILURE, "a tile copy did not complete (TMA wait limit reached)");
  }
}

// The evaluation counters (hypotheses, source windows sampled, of them read
// from staged boxes) into the stats.
static void read_counters(Context& C) {
  unsigned long long ev[3] = {0, 0, 0};
  CK(cudaMemcpy(ev, C.counter.p, sizeof(ev), cudaMemcpyDeviceToHost));
  C.stats.hypotheses_evaluated = ev[0];
  C.stats.windows_evaluated = ev[1];
  C.stats.windows_staged = ev[2];
}

static void finish_stats(Context& C) {
  float ms = 0.f, sw = 0.f;
  if (cudaEventElapsedTime(&ms, C.ev_start, C.ev_end) == cudaSuccess) C.stats.last_run_ms = ms;
  if (cudaEventElapsedTime(&sw, C.ev_sweep0, C.ev_sweep1) == cudaSuccess) C.stats.last_sweep_ms = sw;
  cudaGetLastError();
}

// Device -> pageable host copy through two pinned chunks: the DMA of one
// chunk overlaps the host copy of the previous one (a direct copy into
// pageable memory runs at a fraction of the link's rate).  Synchronous.
static void copy_to_host(Context& C, void* dst, const void* src, size_t bytes) {
  constexpr size_t kChunk = (size_t)8 << 20;
  if (bytes <= ((size_t)1 << 16)) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
    return;
  }
  for (auto& b : C.d2h_buf) b.alloc(kChunk);
  const char* s = static_cast<const char*>(src);
  char* d = static_cast<char*>(dst);
  auto issue = [&](int k, size_t off) {
    const size_t n = std::min(kChunk, bytes - off);
    CK(cudaMemcpyAsync(C.d2h_buf[k].p, s + off, n, cudaMemcpyDeviceToHost, C.stream));
    CK(cudaEventRecord(C.d2h_done[k], C.stream));
  };
  issue(0, 0);
  int k = 0;
  for (size_t off = 0; off < bytes;) {
    const size_t n = std::min(kChunk, bytes - off);
    if (off + n < bytes) issue(k ^ 1, off + n);  // chunk k ^ 1 was copied out last round
    CK(cudaEventSynchronize(C.d2h_done[k]));
    std::memcpy(d + off, C.d2h_buf[k].p, n);
    off += n;
    k ^= 1;
  }
}

static void download_job(Context& C, JobData& D, recon_mvs_depth_map* out, uint32_t* filled) {
  if (!out || !out->depth || !out->support_count || !out->confidence)
    fail(RECON_ERR_INVALID_ARGUMENT, "output depth map arrays NULL");
  if (out->width != D.w || out->height != D.h) fail(RECON_ERR_INVALID_ARGUMENT, "output depth map size mismatch");
  const size_t npx = (size_t)D.w * D.h;
  if (!D.ran) fail(RECON_ERR_INVALID_ARGUMENT, "job has not run");
  if (D.degenerate) {
    CK(cudaStreamSynchronize(C.stream));
    const float nan = std::nanf("");
    std::fill(out->depth, out->depth + npx, nan);
    std::memset(out->support_count, 0, npx);
    std::fill(out->confidence, out->confidence + npx, 0.0f);
    if (out->normal) std::fill(out->normal, out->normal + 3 * npx, 0.0f);
    if (out->cost) std::fill(out->cost, out->cost + npx, 1e30f);
    if (filled) *filled = 0;
    return;
  }
  copy_to_host(C, out->depth, D.out_depth.p, npx * sizeof(float));
  copy_to_host(C, out->support_count, D.out_support.p, npx);
  copy_to_host(C, out->confidence, D.out_conf.p, npx * sizeof(float));
  if (out->normal) {
    if (D.out_normal.p)
      copy_to_host(C, out->normal, D.out_normal.p, 3 * npx * sizeof(float));
    else
      std::fill(out->normal, out->normal + 3 * npx, 0.0f);
  }
  if (out->cost) copy_to_host(C, out->cost, D.out_cost.p, npx * sizeof(float));
  unsigned int f = 0;
  CK(cudaMemcpyAsync(&f, D.filled.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaStreamSynchronize(C.stream));
  check_device_error(C);
  finish_stats(C);
  read_counters(C);
  if (filled) *filled = f;
}

// ---------------------------------------------------------------------------
// default per-thread contexts for the stateless entry points
// ---------------------------------------------------------------------------
static Context& default_context(const recon_mvs_options* opts) {
  thread_local std::map<std::string, std::unique_ptr<Context>> ctxs;
  recon_mvs_options o;
  if (opts)
    o = *opts;
  else
    fill_defaults(&o);
  const std::string key((const char*)&o, sizeof(o));
  auto it = ctxs.find(key);
  if (it == ctxs.end()) it = ctxs.emplace(key, std::make_unique<Context>(o)).first;
  return *it->second;
}

struct JobScope {
  Context& C;
  int id;
  ~JobScope() { erase_job(C, id); }
};

// ---------------------------------------------------------------------------
// parameter registry (params.cpp:386-422) and the StageMvs mapping
// (orchestrator.cpp:952-970)
// ---------------------------------------------------------------------------
enum class PType { kInt, kDouble };
struct PSpec {
  const char* key;
  PType type;
  double def, fast, std_, high, lo, hi;
};
static const PSpec kSpecs[] = {
    {"mvs_patch_size", PType::kInt, 7, 7, 7, 11, 3, 21},
    {"mvs_patch_iterations", PType::kInt, 3, 3, 3, 6, 1, 20},
    {"mvs_patch_random_search_radius", PType::kInt, 2, 2, 2, 4, 0, 16},
    {"mvs_num_views", PType::kInt, 5, 5, 5, 8, 2, 32},
    {"mvs_subpixel_iterations", PType::kInt, 3, 2, 3, 5, 0, 10},
    {"mvs_geo_consistency_threshold", PType::kDouble, 0.02, 0.02, 0.02, 0.01, 0.001, 0.20},
    {"mvs_photo_threshold", PType::kDouble, 0.2, 0.2, 0.2, 0.1, 0.01, 1.0},
    {"mvs_fusion_voxel_size_m", PType::kDouble, 0.001, 0.002, 0.001, 0.0005, 0.0002, 0.005},
    {"mvs_image_scale", PType::kDouble, 1.0, 1.0, 1.0, 1.0, 0.25, 1.0},
    {"mvs_min_depth_m", PType::kDouble, 0.10, 0.10, 0.10, 0.10, 0.02, 1.0},
    {"mvs_max_depth_m", PType::kDouble, 1.50, 1.50, 1.50, 2.00, 0.2, 5.0},
    {"mvs_gpu_tile_size", PType::kInt, 256, 256, 256, 128, 32, 1024},
    {"mvs_pm_search_radius_ratio", PType::kDouble, 0.30, 0.40, 0.30, 0.22, 0.01, 1.0},
    {"mvs_subpixel_window_ratio", PType::kDouble, 0.50, 0.70, 0.50, 0.35, 0.05, 4.0},
    {"mvs_num_threads", PType::kInt, 0, 0, 0, 0, 0, 64},
    // not an mvs_* key, but StageMvs takes num_threads from it (:970)
    {"perf_thread_pool_size", PType::kInt, 0, 0, 0, 0, 0, 64},
};

static void apply_mapped(recon_mvs_config* c, const std::string& key, double v) {
  if (key == "mvs_num_views") c->num_views = (int32_t)v;
  else if (key == "mvs_photo_threshold") c->photo_threshold = v;
  else if (key == "mvs_geo_consistency_threshold") c->geo_consistency_threshold = v;
  // StageMvs feeds the integer radius key into the ratio field (:959-960)
  else if (key == "mvs_patch_random_search_radius") c->random_search_radius_ratio = v;
  else if (key == "mvs_patch_size") c->patch_size = (int32_t)v;
  else if (key == "mvs_patch_iterations") c->iterations = (int32_t)v;
  else if (key == "mvs_subpixel_iterations") c->subpixel_iterations = (int32_t)v;
  else if (key == "mvs_min_depth_m") c->min_depth_m = v;
  else if (key == "mvs_max_depth_m") c->max_depth_m = v;
  else if (key == "mvs_fusion_voxel_size_m") c->fusion_voxel_size_m = v;
  else if (key == "perf_thread_pool_size") c->num_threads = (int32_t)v;
  // registered but not read by StageMvs: mvs_image_scale, mvs_gpu_tile_size,
  // mvs_pm_search_radius_ratio, mvs_subpixel_window_ratio, mvs_num_threads
}

}  // namespace rmvs

using namespace rmvs;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

RECON_API uint32_t recon_mvs_abi_version(void) { return RECON_MVS_GB300_ABI_VERSION; }

RECON_API const char* recon_mvs_last_error(void) { return g_last_error.c_str(); }

RECON_API void recon_mvs_config_default(recon_mvs_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->num_views = 7;
  c->ref_view_index = -1;
  c->ideal_angle_min_deg = 8.0;
  c->ideal_angle_max_deg = 35.0;
  c->max_view_scale_mismatch = 0.15;
  c->view_angle_weight = 1.0;
  c->view_texture_weight = 0.8;
  c->view_spread_weight = 0.6;
  c->view_scale_weight = 0.4;
  c->reference_depth_m = 0.40;
  c->patch_size = 11;
  c->iterations = 4;
  c->random_search_count = 5;
  c->random_search_radius_ratio = 0.30;
  c->restart_ratio = 0.05;
  c->propagation_directions = 4;
  c->propagation_enabled = 1;
  c->num_threads = 0;
  c->photo_threshold = 1.0;
  c->depth_regularization = 0.02;
  c->geo_consistency_threshold = 0.02;
  c->weak_texture_variance = 12.0;
  c->subpixel_iterations = 4;
  c->subpixel_fit_points = 5;
  c->subpixel_window_ratio = 0.005;
  c->min_depth_m = 0.10;
  c->max_depth_m = 1.50;
  c->min_view_consistency = 2;
  c->fusion_voxel_size_m = 0.001;
}

RECON_API void recon_mvs_options_default(recon_mvs_options* o) {
  if (o) fill_defaults(o);
}

RECON_API recon_status recon_mvs_config_set_param(recon_mvs_config* cfg, const char* key, int32_t value_int,
                                                  double value_double) {
  return guard([&] {
    if (!cfg || !key) fail(RECON_ERR_INVALID_ARGUMENT, "NULL config or key");
    const PSpec* spec = nullptr;
    for (const auto& s : kSpecs)
      if (std::strcmp(s.key, key) == 0) spec = &s;
    if (!spec) fail(RECON_ERR_INVALID_ARGUMENT, std::string("unknown parameter ") + key);
    double v = spec->type == PType::kDouble ? value_double : (double)value_int;
    if (std::isnan(v) || std::isinf(v)) v = spec->lo;
    v = std::min(std::max(v, spec->lo), spec->hi);
    if (spec->type == PType::kInt) v = std::nearbyint(v);
    apply_mapped(cfg, key, v);
  });
}

RECON_API recon_status recon_mvs_config_apply_preset(recon_mvs_config* cfg, int32_t preset) {
  return guard([&] {
    if (!cfg || preset < 0 || preset > 2) fail(RECON_ERR_INVALID_ARGUMENT, "bad preset");
    for (const auto& s : kSpecs) {
      const double v = preset == 0 ? s.fast : (preset == 1 ? s.std_ : s.high);
      apply_mapped(cfg, s.key, v);
    }
  });
}

RECON_API recon_status recon_mvs_select_source_views(const recon_pose* ref_pose, const recon_pose* poses,
                                                     int32_t num_poses, const recon_camera_intrinsics* intr,
                                                     const recon_mvs_config* cfg, int32_t* out_indices,
                                                     int32_t capacity, int32_t* out_count) {
  return guard([&] {
    (void)intr;
    if (!ref_pose || (!poses && num_poses > 0) || !cfg || !out_count) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    struct Cand {
      int index;
      double score;
    };
    std::vector<Cand> cands;
    double rc[3];
    center_world(*ref_pose, rc);
    const double kPi = 3.14159265358979323846;
    for (int i = 0; i < num_poses; ++i) {
      if (i == cfg->ref_view_index) continue;
      double sc[3], base[3];
      center_world(poses[i], sc);
      for (int q = 0; q < 3; ++q) base[q] = sc[q] - rc[q];
      double bl = 0.0;
      for (int q = 0; q < 3; ++q) bl += base[q] * base[q];
      if (std::sqrt(bl) < 1e-6) continue;
      const double z_ref = cfg->reference_depth_m;
      const double z_src = z_ref + base[2];
      if (z_src <= 1e-6) continue;
      if (std::fabs(z_ref / z_src - 1.0) > cfg->max_view_scale_mismatch) continue;
      double rel[3];
      for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int q = 0; q < 3; ++q) s += ref_pose->r[r * 3 + q] * base[q];
        rel[r] = s;
      }
      double dd = 0.0;
      for (int q = 0; q < 3; ++q) dd += rel[q] * rel[q];
      const double dist = std::sqrt(dd);
      if (dist < 1e-6) continue;
      const double angle = std::acos(std::clamp(rel[2] / dist, -1.0, 1.0)) * 180.0 / kPi;
      double score;
      if (angle < cfg->ideal_angle_min_deg)
        score = angle / cfg->ideal_angle_min_deg;
      else if (angle > cfg->ideal_angle_max_deg)
        score = std::max(0.0, 1.0 - (angle - cfg->ideal_angle_max_deg) / (cfg->ideal_angle_max_deg * 2.0));
      else
        score = 1.0;
      cands.push_back({i, score * cfg->view_angle_weight});
    }
    // the same library sort as the reference (:194-197)
    std::sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.score > b.score; });
    int n = 0;
    for (size_t i = 0; i < cands.size() && n < cfg->num_views; ++i) {
      if (out_indices && n < capacity) out_indices[n] = cands[i].index;
      ++n;
    }
    *out_count = std::min(n, std::max(0, capacity));
  });
}

RECON_API recon_status recon_mvs_compute_ncc(const uint8_t* ref, int32_t ref_w, int32_t ref_h, const uint8_t* src,
                                             int32_t src_w, int32_t src_h, const double* coords, int32_t n,
                                             int32_t patch_size, recon_mvs_ncc_result* out) {
  return guard([&] {
    if (!ref || !src || (!coords && n > 0) || (!out && n > 0)) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    check_image_size(ref_w, ref_h, "reference");
    check_image_size(src_w, src_h, "source");
    if (n < 0) fail(RECON_ERR_INVALID_ARGUMENT, "negative window count");
    if (n == 0) return;
    Context& C = default_context(nullptr);
    C.use();
    DevArray<uint8_t> dr, ds;
    DevArray<NccWindow> dw;
    DevArray<int> dv, dk, dn;
    DevArray<double> dc;
    dr.alloc((size_t)ref_w * ref_h);
    ds.alloc((size_t)src_w * src_h);
    dw.alloc(n);
    dv.alloc(n);
    dk.alloc(n);
    dn.alloc(n);
    dc.alloc(n);
    CK(cudaMemcpyAsync(dr.p, ref, (size_t)ref_w * ref_h, cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(ds.p, src, (size_t)src_w * src_h, cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(dw.p, coords, sizeof(NccWindow) * n, cudaMemcpyHostToDevice, C.stream));
    CK(launch_ncc_windows(dr.p, ref_w, ref_h, ds.p, src_w, src_h, patch_size, n, dw.p, dv.p, dc.p, dk.p, dn.p,
                          C.stream));
    std::vector<int> v(n), k(n), s(n);
    std::vector<double> c(n);
    CK(cudaMemcpyAsync(v.data(), dv.p, n * sizeof(int), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(k.data(), dk.p, n * sizeof(int), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(s.data(), dn.p, n * sizeof(int), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(c.data(), dc.p, n * sizeof(double), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
    for (int i = 0; i < n; ++i) out[i] = recon_mvs_ncc_result{v[i], c[i], k[i], s[i]};
  });
}

RECON_API recon_status recon_mvs_evaluate(const recon_mvs_views* views, const recon_mvs_config* cfg,
                                          const recon_mvs_options* opts, int32_t n, const int32_t* px,
                                          const int32_t* py, const double* inv_depth, const float* normals,
                                          float* out_cost, int32_t* out_support, float* out_view_cost) {
  return guard([&] {
    if (n < 0 || (n > 0 && (!px || !py || !inv_depth || !out_cost || !out_support)))
      fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    Context& C = default_context(opts);
    const bool plane = C.opts.mode == RECON_MVS_MODE_PLANE;
    if (plane && n > 0 && !normals) fail(RECON_ERR_INVALID_ARGUMENT, "plane mode needs normals");
    const int id = stage_job(C, views, cfg, false, nullptr, 0);
    JobScope scope{C, id};
    if (n == 0) return;
    JobData& D = get_job(C, id);
    for (int i = 0; i < n; ++i)
      if (px[i] < 0 || py[i] < 0 || px[i] >= D.w || py[i] >= D.h) fail(RECON_ERR_INVALID_ARGUMENT, "pixel outside image");
    DevArray<int> dx, dy, ds;
    DevArray<double> di;
    DevArray<float> dn, dc, dv;
    dx.alloc(n);
    dy.alloc(n);
    ds.alloc(n);
    di.alloc(n);
    dc.alloc(n);
    CK(cudaMemcpyAsync(dx.p, px, n * sizeof(int), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(dy.p, py, n * sizeof(int), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(di.p, inv_depth, n * sizeof(double), cudaMemcpyHostToDevice, C.stream));
    if (plane) {
      dn.alloc((size_t)n * 3);
      CK(cudaMemcpyAsync(dn.p, normals, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, C.stream));
    }
    if (out_view_cost) dv.alloc((size_t)n * D.num_src);
    CK(launch_eval_hyps(D.J, plane ? 1 : 0, n, dx.p, dy.p, di.p, dn.p, dc.p, ds.p, out_view_cost ? dv.p : nullptr,
                        C.stream));
    CK(cudaMemcpyAsync(out_cost, dc.p, n * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(out_support, ds.p, n * sizeof(int), cudaMemcpyDeviceToHost, C.stream));
    if (out_view_cost)
      CK(cudaMemcpyAsync(out_view_cost, dv.p, (size_t)n * D.num_src * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
  });
}

// ---- the differentiation form ---------------------------------------------
static void check_hyps(const JobData& D, int n, const int32_t* px, const int32_t* py, const double* depth,
                       const double* angles) {
  if (n < 0 || (n > 0 && (!px || !py || !depth || !angles))) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
  if (D.opts.mode != RECON_MVS_MODE_PLANE) fail(RECON_ERR_INVALID_ARGUMENT, "the adjoint needs a plane-mode job");
  if (D.num_src > kMaxSources) fail(RECON_ERR_INVALID_ARGUMENT, "more than 32 sources");
  for (int i = 0; i < n; ++i)
    if (px[i] < 0 || py[i] < 0 || px[i] >= D.w || py[i] >= D.h) fail(RECON_ERR_INVALID_ARGUMENT, "pixel outside image");
}

struct HypUpload {
  DevArray<int> x, y;
  DevArray<double> d, a;
  void put(Context& C, int n, const int32_t* px, const int32_t* py, const double* depth, const double* angles) {
    x.alloc(n);
    y.alloc(n);
    d.alloc(n);
    a.alloc((size_t)2 * n);
    CK(cudaMemcpyAsync(x.p, px, n * sizeof(int), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(y.p, py, n * sizeof(int), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(d.p, depth, n * sizeof(double), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(a.p, angles, (size_t)2 * n * sizeof(double), cudaMemcpyHostToDevice, C.stream));
  }
};

RECON_API recon_status recon_mvs_job_adjoint(void* ctx, int32_t job, int32_t n, const int32_t* px, const int32_t* py,
                                             const double* depth, const double* angles, float* out_cost,
                                             float* out_grad, float* out_gn, float* out_pose_grad) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    JobData& D = get_job(C, job);
    check_hyps(D, n, px, py, depth, angles);
    if (n > 0 && (!out_cost || !out_grad)) fail(RECON_ERR_INVALID_ARGUMENT, "NULL output");
    if (n == 0) return;
    HypUpload U;
    U.put(C, n, px, py, depth, angles);
    DevArray<float> dc, dg, dh, dp;
    dc.alloc(n);
    dg.alloc((size_t)3 * n);
    if (out_gn) dh.alloc((size_t)6 * n);
    if (out_pose_grad) dp.alloc((size_t)6 * n * D.num_src);
    CK(launch_plane_adjoint(D.J, n, U.x.p, U.y.p, U.d.p, U.a.p, dc.p, dg.p, out_gn ? dh.p : nullptr,
                            out_pose_grad ? dp.p : nullptr, C.stream));
    CK(cudaMemcpyAsync(out_cost, dc.p, n * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(out_grad, dg.p, (size_t)3 * n * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    if (out_gn) CK(cudaMemcpyAsync(out_gn, dh.p, (size_t)6 * n * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    if (out_pose_grad)
      CK(cudaMemcpyAsync(out_pose_grad, dp.p, (size_t)6 * n * D.num_src * sizeof(float), cudaMemcpyDeviceToHost,
                         C.stream));
    CK(cudaStreamSynchronize(C.stream));
  });
}

// Rodrigues: R = exp([w]x), FP64.
static void so3_exp(const double w[3], double R[9]) {
  const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  const double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double a, b;
  if (th < 1e-12) {
    a = 1.0;
    b = 0.5;
  } else {
    a = std::sin(th) / th;
    b = (1.0 - std::cos(th)) / (th * th);
  }
  double K2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = 0.0;
      for (int q = 0; q < 3; ++q) t += K[i * 3 + q] * K[q * 3 + j];
      K2[i * 3 + j] = t;
    }
  for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0 ? 1.0 : 0.0) + a * K[i] + b * K2[i];
}

// Left perturbation of a world -> camera pose in the camera frame:
// R' = exp([w]x) R, t' = exp([w]x) t + tau.
static recon_pose perturb_pose(const recon_pose& p, const double w[3], const double tau[3]) {
  double E[9];
  so3_exp(w, E);
  recon_pose q = p;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      double t = 0.0;
      for (int k = 0; k < 3; ++k) t += E[i * 3 + k] * p.r[k * 3 + j];
      q.r[i * 3 + j] = t;
    }
    double t = 0.0;
    for (int k = 0; k < 3; ++k) t += E[i * 3 + k] * p.t[k];
    q.t[i] = t + tau[i];
  }
  return q;
}

// Solves (H + lambda diag(H)) x = -g for symmetric positive 6 x 6 H given as
// its upper triangle (row-major order), by Cholesky in FP64.
static bool solve_lm6(const double* Hu, const double* g, double lambda, double x[6]) {
  double M[36];
  int t = 0;
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j, ++t) M[i * 6 + j] = M[j * 6 + i] = Hu[t];
  for (int i = 0; i < 6; ++i) M[i * 6 + i] *= 1.0 + lambda;
  double L[36] = {0};
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = M[i * 6 + j];
      for (int k = 0; k < j; ++k) s -= L[i * 6 + k] * L[j * 6 + k];
      if (i == j) {
        if (!(s > 0.0)) return false;
        L[i * 6 + i] = std::sqrt(s);
      } else {
        L[i * 6 + j] = s / L[j * 6 + j];
      }
    }
  double y[6];
  for (int i = 0; i < 6; ++i) {
    double s = -g[i];
    for (int k = 0; k < i; ++k) s -= L[i * 6 + k] * y[k];
    y[i] = s / L[i * 6 + i];
  }
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < 6; ++k) s -= L[k * 6 + i] * x[k];
    x[i] = s / L[i * 6 + i];
  }
  for (int i = 0; i < 6; ++i)
    if (!std::isfinite(x[i])) return false;
  return true;
}

// Per-source sums of the pose normal equations over the hypotheses.
struct PoseSums {
  std::vector<double> cost, count, g, H;  // per source: 1, 1, 6, 21
};

static PoseSums pose_normal_eq(Context& C, JobData& D, const HypUpload& U, int n, DevArray<float>& part) {
  const int rec = pose_partial_records();
  const int blocks = (n + 127) / 128;
  const int S = D.num_src;
  part.alloc((size_t)blocks * S * rec);
  CK(launch_pose_normal_eq(D.J, n, U.x.p, U.y.p, U.d.p, U.a.p, part.p, C.stream));
  std::vector<float> host((size_t)blocks * S * rec);
  CK(cudaMemcpyAsync(host.data(), part.p, host.size() * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaStreamSynchronize(C.stream));
  PoseSums P;
  P.cost.assign(S, 0.0);
  P.count.assign(S, 0.0);
  P.g.assign((size_t)S * 6, 0.0);
  P.H.assign((size_t)S * 21, 0.0);
  for (int b = 0; b < blocks; ++b)
    for (int s = 0; s < S; ++s) {
      const float* r = &host[((size_t)b * S + s) * rec];
      P.cost[s] += r[0];
      for (int i = 0; i < 6; ++i) P.g[(size_t)s * 6 + i] += r[1 + i];
      for (int i = 0; i < 21; ++i) P.H[(size_t)s * 21 + i] += r[7 + i];
      P.count[s] += r[28];
    }
  return P;
}

static void upload_src_table(Context& C, JobData& D) {
  CK(cudaMemcpyAsync(D.src_table.p, D.host_src.data(), sizeof(SrcView) * D.num_src, cudaMemcpyHostToDevice,
                     C.stream));
  CK(cudaStreamSynchronize(C.stream));
}

RECON_API recon_status recon_mvs_job_recover_poses(void* ctx, int32_t job, int32_t n, const int32_t* px,
                                                   const int32_t* py, const double* depth, const double* angles,
                                                   int32_t iterations, recon_pose* out_src_poses,
                                                   double* out_cost) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    if (iterations < 0) fail(RECON_ERR_INVALID_ARGUMENT, "iterations < 0");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    JobData& D = get_job(C, job);
    check_hyps(D, n, px, py, depth, angles);
    if (D.degenerate) fail(RECON_ERR_INVALID_ARGUMENT, "degenerate job");
    if (C.plan && std::find(C.plan->ids.begin(), C.plan->ids.end(), job) != C.plan->ids.end()) {
      CK(cudaStreamSynchronize(C.stream));
      C.plan.reset();  // the captured launches carry the job's old transforms
    }
    const int S = D.num_src;
    HypUpload U;
    U.put(C, n, px, py, depth, angles);
    DevArray<float> part;
    auto mean = [](const PoseSums& P, int s) { return P.count[s] > 0 ? P.cost[s] / P.count[s] : 1e30; };
    PoseSums cur = pose_normal_eq(C, D, U, n, part);
    auto total = [&](const PoseSums& P) {
      double t = 0.0;
      for (int s = 0; s < S; ++s) t += mean(P, s);
      return t;
    };
    if (out_cost) out_cost[0] = total(cur);
    std::vector<double> lambda(S, 1e-4);
    for (int it = 0; it < iterations; ++it) {
      std::vector<recon_pose> prev = D.src_pose;
      std::vector<bool> moved(S, false);
      for (int s = 0; s < S; ++s) {
        if (cur.count[s] < 6) continue;
        double x[6];
        if (!solve_lm6(&cur.H[(size_t)s * 21], &cur.g[(size_t)s * 6], lambda[s], x)) {
          lambda[s] *= 10.0;
          continue;
        }
        D.src_pose[s] = perturb_pose(prev[s], x, x + 3);
        set_src_transform(D.host_src[s], D.ref_pose, D.src_pose[s], D.ref_intr);
        moved[s] = true;
      }
      upload_src_table(C, D);
      PoseSums trial = pose_normal_eq(C, D, U, n, part);
      for (int s = 0; s < S; ++s) {
        if (!moved[s]) continue;
        if (mean(trial, s) < mean(cur, s)) {
          cur.cost[s] = trial.cost[s];
          cur.count[s] = trial.count[s];
          for (int i = 0; i < 6; ++i) cur.g[(size_t)s * 6 + i] = trial.g[(size_t)s * 6 + i];
          for (int i = 0; i < 21; ++i) cur.H[(size_t)s * 21 + i] = trial.H[(size_t)s * 21 + i];
          lambda[s] *= 0.3;
        } else {
          D.src_pose[s] = prev[s];
          set_src_transform(D.host_src[s], D.ref_pose, D.src_pose[s], D.ref_intr);
          lambda[s] *= 10.0;
        }
      }
      upload_src_table(C, D);
      if (out_cost) out_cost[it + 1] = total(cur);
    }
    if (out_src_poses)
      for (int s = 0; s < S; ++s) out_src_poses[s] = D.src_pose[s];
  });
}

RECON_API recon_status recon_mvs_patchmatch(const recon_mvs_views* views, const recon_mvs_config* cfg,
                                            const recon_mvs_options* opts, const double* seed_points,
                                            int32_t num_seeds, recon_mvs_depth_map* out, uint32_t* out_filled) {
  return guard([&] {
    if (!out) fail(RECON_ERR_INVALID_ARGUMENT, "out is NULL");
    Context& C = default_context(opts);
    const int id = stage_job(C, views, cfg, false, seed_points, num_seeds);
    JobScope scope{C, id};
    run_job(C, id);
    download_job(C, get_job(C, id), out, out_filled);
  });
}

RECON_API recon_status recon_mvs_refine_subpixel(const recon_mvs_views* views, const recon_mvs_config* cfg,
                                                 const recon_mvs_options* opts, recon_mvs_depth_map* depth,
                                                 uint32_t* out_refined) {
  return guard([&] {
    if (!depth || !depth->depth || !depth->confidence) fail(RECON_ERR_INVALID_ARGUMENT, "depth map NULL");
    recon_mvs_options o;
    if (opts)
      o = *opts;
    else
      fill_defaults(&o);
    o.mode = RECON_MVS_MODE_COMPAT;  // RefineSubpixel's cost is the reference's
    Context& C = default_context(&o);
    const int id = stage_job(C, views, cfg, false, nullptr, 0);
    JobScope scope{C, id};
    JobData& D = get_job(C, id);
    if (depth->width != D.w || depth->height != D.h) fail(RECON_ERR_INVALID_ARGUMENT, "depth map size mismatch");
    if (out_refined) *out_refined = 0;
    const double baseline = mean_baseline(*views->ref_pose, views->src_poses, views->source_indices, views->num_src);
    if (baseline < 1e-9) return;  // the reference returns 0 (:786)
    const size_t npx = (size_t)D.w * D.h;
    CK(cudaMemcpyAsync(D.out_depth.p, depth->depth, npx * sizeof(float), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemcpyAsync(D.out_conf.p, depth->confidence, npx * sizeof(float), cudaMemcpyHostToDevice, C.stream));
    CK(cudaMemsetAsync(D.filled.p, 0, sizeof(unsigned int), C.stream));
    CK(launch_compat_refine(D.J, D.out_depth.p, D.out_conf.p, D.inv_per_px, cfg->subpixel_fit_points,
                            cfg->subpixel_iterations, D.filled.p, nullptr, nullptr, C.stream));
    unsigned int f = 0;
    CK(cudaMemcpyAsync(depth->depth, D.out_depth.p, npx * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(depth->confidence, D.out_conf.p, npx * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(&f, D.filled.p, sizeof(f), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
    if (out_refined) *out_refined = f;
  });
}

// One device-resident depth map with its camera (consistency, fusion).
struct DevMap {
  int w, h;
  const float* depth;
  recon_camera_intrinsics intr;
  recon_pose pose;
};

// Geometric consistency of `ref` against `others` on the device: per pixel
// the number of consistent maps (out_count) and count >= min_views (out_keep).
static void consistency_device(Context& C, const DevMap& ref, const std::vector<DevMap>& others, float rel_depth_max,
                               float reproj_px_max, int min_views, uint8_t* out_count, uint8_t* out_keep) {
  ConsistencyRef cr{ref.w, ref.h, ref.depth, (float)ref.intr.fx, (float)ref.intr.fy, (float)ref.intr.cx,
                    (float)ref.intr.cy};
  std::vector<ConsistencySrc> srcs;
  for (const DevMap& o : others) {
    srcs.push_back(consistency_source(o.w, o.h, o.depth, o.intr, ref.pose, o.pose));
  }
  DevArray<ConsistencySrc> ds;
  ds.alloc(std::max<size_t>(1, srcs.size()));
  if (!srcs.empty())
    CK(cudaMemcpyAsync(ds.p, srcs.data(), srcs.size() * sizeof(ConsistencySrc), cudaMemcpyHostToDevice, C.stream));
  CK(launch_consistency(cr, ds.p, (int)srcs.size(), rel_depth_max, reproj_px_max, min_views, out_count, out_keep,
                        C.stream));
  CK(cudaStreamSynchronize(C.stream));  // the descriptor table is freed on return
}

RECON_API recon_status recon_mvs_geometric_consistency(const recon_mvs_depth_map* maps, const recon_pose* poses,
                                                       const recon_camera_intrinsics* intr, int32_t num_maps,
                                                       int32_t ref_index, float rel_depth_max, float reproj_px_max,
                                                       int32_t min_views, uint8_t* out_count, uint8_t* out_keep) {
  return guard([&] {
    if (!maps || !poses || !intr || num_maps <= 0 || ref_index < 0 || ref_index >= num_maps || !out_count || !out_keep)
      fail(RECON_ERR_INVALID_ARGUMENT, "bad argument");
    Context& C = default_context(nullptr);
    C.use();
    std::vector<std::unique_ptr<DevArray<float>>> dev(num_maps);
    for (int m = 0; m < num_maps; ++m) {
      dev[m] = std::make_unique<DevArray<float>>();
      const size_t n = map_pixels(maps[m]);
      if (n == 0) continue;
      dev[m]->alloc(n);
      CK(cudaMemcpyAsync(dev[m]->p, maps[m].depth, n * sizeof(float), cudaMemcpyHostToDevice, C.stream));
    }
    const recon_mvs_depth_map& R = maps[ref_index];
    if (map_pixels(R) == 0) fail(RECON_ERR_INVALID_ARGUMENT, "reference map NULL or empty");
    std::vector<DevMap> others;
    for (int s = 0; s < num_maps; ++s)
      if (s != ref_index && dev[s]->p)
        others.push_back(DevMap{maps[s].width, maps[s].height, dev[s]->p, intr[s], poses[s]});
    const size_t n = (size_t)R.width * R.height;
    DevArray<uint8_t> dc, dk;
    dc.alloc(n);
    dk.alloc(n);
    consistency_device(C, DevMap{R.width, R.height, dev[ref_index]->p, intr[ref_index], poses[ref_index]}, others,
                       rel_depth_max, reproj_px_max, min_views, dc.p, dk.p);
    CK(cudaMemcpyAsync(out_count, dc.p, n, cudaMemcpyDeviceToHost, C.stream));
    CK(cudaMemcpyAsync(out_keep, dk.p, n, cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
  });
}

RECON_API void recon_mvs_point_cloud_free(recon_mvs_point_cloud* c) {
  if (!c) return;
  std::free(c->positions);
  std::free(c->normals);
  std::free(c->colors);
  std::free(c->confidences);
  std::free(c->keys);
  std::free(c->counts);
  std::memset(c, 0, sizeof(*c));
}

static FuseMap fuse_map(int w, int h, const float* depth, const uint8_t* support, const float* conf,
                        const uint8_t* keep, const recon_camera_intrinsics& k, const recon_pose& pose,
                        const float* normal = nullptr) {
  FuseMap M;
  std::memset(&M, 0, sizeof(M));
  M.normal = normal;
  M.w = w;
  M.h = h;
  M.depth = depth;
  M.support = support;
  M.conf = conf;
  M.keep = keep;
  M.fx = k.fx;
  M.fy = k.fy;
  M.cx = k.cx;
  M.cy = k.cy;
  M.k1 = k.k1;
  M.k2 = k.k2;
  M.k3 = k.k3;
  M.p1 = k.p1;
  M.p2 = k.p2;
  for (int i = 0; i < 9; ++i) M.R[i] = pose.r[i];
  for (int i = 0; i < 3; ++i) M.t[i] = pose.t[i];
  return M;
}

// A fused cloud in device memory: one record per voxel, in the order of the
// voxels' first points.
struct DevCloud {
  unsigned int n = 0;
  DevArray<unsigned long long> key;
  DevArray<double> pos, nrm;
  DevArray<float> conf;
  DevArray<unsigned int> cnt;
};

// FuseDepthMaps on device-resident maps (FuseMap: device pointers, camera):
// the reference's voxel keys in FP64, a hash table of first occurrences,
// buckets of points per voxel in the reference's insertion order, sequential
// FP64 sums.  The cloud stays in device memory (`out`).
static void fuse_maps_device(Context& C, const std::vector<FuseMap>& maps, const recon_mvs_config& cfg,
                             DevCloud* out) {
  out->n = 0;
  if (maps.empty() || cfg.fusion_voxel_size_m <= 0.0) return;
  int64_t total = 0;
  std::vector<int64_t> base(maps.size());
  for (size_t m = 0; m < maps.size(); ++m) {
    base[m] = total;
    total += (int64_t)maps[m].w * maps[m].h;
  }
  if (total == 0) return;
  DevArray<unsigned long long> key, tkey, tfirst;
  DevArray<double> pos, nrm;
  DevArray<float> conf;
  DevArray<uint8_t> valid;
  DevArray<int> slot_of, err;
  DevArray<unsigned int> tcount, flag, vid_of, slot_vid, scratch;
  key.alloc(total);
  pos.alloc(3 * total);
  nrm.alloc(3 * total);
  conf.alloc(total);
  valid.alloc(total);
  slot_of.alloc(total);
  flag.alloc(total);
  vid_of.alloc(total);
  err.alloc(1);
  uint64_t cap = 1024;
  while (cap < 2 * (uint64_t)total) cap <<= 1;
  if (cap > (1ull << 30)) fail(RECON_ERR_INVALID_ARGUMENT, "more pixels than one fusion call can key (2^29)");
  // cap probed slots + the side slot of the one key equal to the empty marker
  tkey.alloc(cap);
  tfirst.alloc(cap + 1);
  tcount.alloc(cap + 1);
  slot_vid.alloc(cap + 1);
  CK(cudaMemsetAsync(tkey.p, 0x7F, cap * sizeof(unsigned long long), C.stream));
  CK(cudaMemsetAsync(tfirst.p, 0xFF, (cap + 1) * sizeof(unsigned long long), C.stream));
  CK(cudaMemsetAsync(tcount.p, 0, (cap + 1) * sizeof(unsigned int), C.stream));
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), C.stream));
  const FuseParams P{cfg.fusion_voxel_size_m, cfg.photo_threshold, cfg.min_view_consistency};
  for (size_t m = 0; m < maps.size(); ++m)
    CK(launch_fuse_points(maps[m], base[m], P, key.p, pos.p, nrm.p, conf.p, valid.p, C.stream));
  CK(cudaMemsetAsync(slot_of.p, 0xFF, total * sizeof(int), C.stream));  // -1: no slot
  CK(launch_fuse_insert(total, key.p, valid.p, tkey.p, tcount.p, tfirst.p, cap - 1, slot_of.p, err.p, C.stream));
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaStreamSynchronize(C.stream));
  if (herr) fail(RECON_ERR_INTERNAL, "voxel hash table overflow");
  CK(launch_fuse_flags(total, valid.p, slot_of.p, tfirst.p, flag.p, C.stream));
  scratch.alloc(scan_scratch_elems(total));
  CK(exclusive_scan_u32(flag.p, vid_of.p, total, scratch.p, C.stream));
  unsigned int last_vid = 0, last_flag = 0;
  CK(cudaMemcpyAsync(&last_vid, vid_of.p + total - 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemcpyAsync(&last_flag, flag.p + total - 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaStreamSynchronize(C.stream));
  const unsigned int nvox = last_vid + last_flag;
  if (nvox == 0) return;
  DevArray<unsigned int> vcount, voffset, cursor;
  vcount.alloc(nvox);
  voffset.alloc(nvox);
  cursor.alloc(nvox);
  CK(launch_fuse_voxels(total, flag.p, vid_of.p, slot_of.p, tcount.p, slot_vid.p, vcount.p, C.stream));
  scratch.alloc(std::max<int64_t>(scan_scratch_elems(nvox), (int64_t)scratch.n));
  CK(exclusive_scan_u32(vcount.p, voffset.p, nvox, scratch.p, C.stream));
  unsigned int last_off = 0, last_cnt = 0;
  CK(cudaMemcpyAsync(&last_off, voffset.p + nvox - 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemcpyAsync(&last_cnt, vcount.p + nvox - 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemsetAsync(cursor.p, 0, nvox * sizeof(unsigned int), C.stream));
  CK(cudaStreamSynchronize(C.stream));
  const int64_t npts = (int64_t)last_off + last_cnt;
  DevArray<int64_t> bucket;
  bucket.alloc(npts);
  CK(launch_fuse_scatter(total, valid.p, slot_of.p, slot_vid.p, voffset.p, cursor.p, bucket.p, C.stream));
  out->key.alloc(nvox);
  out->pos.alloc(3 * (size_t)nvox);
  out->nrm.alloc(3 * (size_t)nvox);
  out->conf.alloc(nvox);
  out->cnt.alloc(nvox);
  CK(launch_fuse_reduce(nvox, voffset.p, vcount.p, bucket.p, key.p, pos.p, nrm.p, conf.p, out->key.p, out->pos.p,
                        out->nrm.p, out->conf.p, out->cnt.p, C.stream));
  CK(cudaStreamSynchronize(C.stream));  // the working arrays are freed on return
  out->n = nvox;
}

// The same, with the cloud copied into malloc-allocated host arrays
// (recon_mvs_point_cloud_free).
static void download_cloud(Context& C, const DevCloud& dc, recon_mvs_point_cloud* out) {
  std::memset(out, 0, sizeof(*out));
  const unsigned int nvox = dc.n;
  if (nvox == 0) return;
  out->count = nvox;
  out->positions = (double*)std::malloc(3 * sizeof(double) * nvox);
  out->normals = (double*)std::malloc(3 * sizeof(double) * nvox);
  out->colors = (float*)std::calloc(3 * (size_t)nvox, sizeof(float));
  out->confidences = (float*)std::malloc(sizeof(float) * nvox);
  out->keys = (int64_t*)std::malloc(sizeof(int64_t) * nvox);
  out->counts = (uint32_t*)std::malloc(sizeof(uint32_t) * nvox);
  if (!out->positions || !out->normals || !out->colors || !out->confidences || !out->keys || !out->counts) {
    recon_mvs_point_cloud_free(out);
    fail(RECON_ERR_OUT_OF_MEMORY, "point cloud allocation failed");
  }
  CK(cudaMemcpyAsync(out->positions, dc.pos.p, 3 * sizeof(double) * nvox, cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemcpyAsync(out->normals, dc.nrm.p, 3 * sizeof(double) * nvox, cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemcpyAsync(out->confidences, dc.conf.p, sizeof(float) * nvox, cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemcpyAsync(out->keys, dc.key.p, sizeof(int64_t) * nvox, cudaMemcpyDeviceToHost, C.stream));
  CK(cudaMemcpyAsync(out->counts, dc.cnt.p, sizeof(uint32_t) * nvox, cudaMemcpyDeviceToHost, C.stream));
  CK(cudaStreamSynchronize(C.stream));
}

static void fuse_maps(Context& C, const std::vector<FuseMap>& maps, const recon_mvs_config& cfg,
                      recon_mvs_point_cloud* out) {
  DevCloud dc;
  fuse_maps_device(C, maps, cfg, &dc);
  download_cloud(C, dc, out);

}

RECON_API recon_status recon_mvs_fuse(const recon_mvs_depth_map* maps, const recon_pose* poses,
                                      const recon_camera_intrinsics* intr, int32_t num_maps,
                                      const recon_mvs_config* cfg, const uint8_t* const* keep_masks,
                                      recon_mvs_point_cloud* out) {
  return guard([&] {
    if (!out || !cfg) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    if (num_maps <= 0) return;
    if (!maps || !poses || !intr) fail(RECON_ERR_INVALID_ARGUMENT, "NULL maps/poses/intrinsics");
    if (cfg->fusion_voxel_size_m <= 0.0) return;
    Context& C = default_context(nullptr);
    C.use();
    std::vector<std::unique_ptr<DevArray<float>>> dd, dc;
    std::vector<std::unique_ptr<DevArray<uint8_t>>> dsup, dkeep;
    std::vector<FuseMap> fm;
    for (int m = 0; m < num_maps; ++m) {
      const size_t n = map_pixels(maps[m]);
      if (n == 0) continue;
      if (!maps[m].support_count || !maps[m].confidence) fail(RECON_ERR_INVALID_ARGUMENT, "map arrays NULL");
      dd.push_back(std::make_unique<DevArray<float>>());
      dc.push_back(std::make_unique<DevArray<float>>());
      dsup.push_back(std::make_unique<DevArray<uint8_t>>());
      dkeep.push_back(std::make_unique<DevArray<uint8_t>>());
      dd.back()->alloc(n);
      dc.back()->alloc(n);
      dsup.back()->alloc(n);
      CK(cudaMemcpyAsync(dd.back()->p, maps[m].depth, n * sizeof(float), cudaMemcpyHostToDevice, C.stream));
      CK(cudaMemcpyAsync(dc.back()->p, maps[m].confidence, n * sizeof(float), cudaMemcpyHostToDevice, C.stream));
      CK(cudaMemcpyAsync(dsup.back()->p, maps[m].support_count, n, cudaMemcpyHostToDevice, C.stream));
      const uint8_t* keep = nullptr;
      if (keep_masks && keep_masks[m]) {
        dkeep.back()->alloc(n);
        CK(cudaMemcpyAsync(dkeep.back()->p, keep_masks[m], n, cudaMemcpyHostToDevice, C.stream));
        keep = dkeep.back()->p;
      }
      fm.push_back(fuse_map(maps[m].width, maps[m].height, dd.back()->p, dsup.back()->p, dc.back()->p, keep,
                            intr[m], poses[m]));
    }
    fuse_maps(C, fm, *cfg, out);
  });
}

RECON_API recon_status recon_mvs_undistort(const uint8_t* img, int32_t w, int32_t h,
                                           const recon_camera_intrinsics* intr, float* out) {
  return guard([&] {
    if (!img || !intr || !out) fail(RECON_ERR_INVALID_ARGUMENT, "bad argument");
    check_image_size(w, h, "undistort");
    Context& C = default_context(nullptr);
    C.use();
    DevArray<uint8_t> di;
    DevArray<float> dout;
    di.alloc((size_t)w * h);
    dout.alloc((size_t)w * h);
    CK(cudaMemcpyAsync(di.p, img, (size_t)w * h, cudaMemcpyHostToDevice, C.stream));
    UndistortCam K{intr->fx, intr->fy, intr->cx, intr->cy, intr->k1, intr->k2, intr->k3, intr->p1, intr->p2};
    CK(launch_undistort(di.p, w, h, K, dout.p, C.stream));
    CK(cudaMemcpyAsync(out, dout.p, (size_t)w * h * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
  });
}

RECON_API recon_status recon_mvs_context_create(const recon_mvs_options* opts, void** out_ctx) {
  return guard([&] {
    if (!out_ctx) fail(RECON_ERR_INVALID_ARGUMENT, "out_ctx NULL");
    recon_mvs_options o;
    if (opts)
      o = *opts;
    else
      fill_defaults(&o);
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (o.device < 0 || o.device >= ndev) fail(RECON_ERR_INVALID_ARGUMENT, "no such CUDA device");
    *out_ctx = new Context(o);
  });
}

RECON_API void recon_mvs_context_destroy(void* ctx) { delete static_cast<Context*>(ctx); }

RECON_API recon_status recon_mvs_job_stage(void* ctx, const recon_mvs_views* views, const recon_mvs_config* cfg,
                                           int32_t undistort, int32_t* out_job) {
  return guard([&] {
    if (!ctx || !out_job) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    *out_job = stage_job(*static_cast<Context*>(ctx), views, cfg, undistort != 0, nullptr, 0);
  });
}

RECON_API recon_status recon_mvs_image_stage(void* ctx, const uint8_t* gray, int32_t w, int32_t h,
                                             const recon_camera_intrinsics* intr, int32_t undistort,
                                             int32_t* out_image) {
  return guard([&] {
    if (!ctx || !intr || !out_image) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    auto I = stage_image(C, gray, w, h, *intr, undistort != 0);
    CK(cudaStreamSynchronize(C.stream));  // the host image may go away after the call
    const int id = C.next_image++;
    C.images[id] = std::move(I);
    *out_image = id;
  });
}

RECON_API recon_status recon_mvs_image_stage_bgra(void* ctx, const uint8_t* bgra, int32_t w, int32_t h,
                                                  int32_t stride, const recon_camera_intrinsics* intr,
                                                  int32_t undistort, int32_t* out_image) {
  return guard([&] {
    if (!ctx || !intr || !out_image) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    auto I = stage_image_bgra(C, bgra, w, h, stride, *intr, undistort != 0);
    const int id = C.next_image++;
    C.images[id] = std::move(I);
    *out_image = id;
  });
}

RECON_API recon_status recon_mvs_bgra_to_gray(const uint8_t* bgra, int32_t w, int32_t h, int32_t stride,
                                              uint8_t* out) {
  return guard([&] {
    check_image_size(w, h, "BGRA");
    if (!bgra || !out || stride < 4 * w) fail(RECON_ERR_INVALID_ARGUMENT, "bad argument");
    Context& C = default_context(nullptr);
    C.use();
    DevArray<uint8_t> dev, g;
    dev.alloc((size_t)4 * w * h);
    g.alloc((size_t)w * h);
    CK(cudaMemcpy2DAsync(dev.p, (size_t)4 * w, bgra, (size_t)stride, (size_t)4 * w, h, cudaMemcpyHostToDevice,
                         C.stream));
    CK(launch_bgra_to_gray(dev.p, w, h, g.p, C.stream));
    CK(cudaMemcpyAsync(out, g.p, (size_t)w * h, cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
  });
}

RECON_API recon_status recon_mvs_image_release(void* ctx, int32_t image) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    if (!C.images.erase(image)) fail(RECON_ERR_INVALID_ARGUMENT, "unknown image id");
  });
}

RECON_API recon_status recon_mvs_job_stage_images(void* ctx, int32_t ref_image, int32_t num_src,
                                                  const int32_t* src_images, const recon_pose* ref_pose,
                                                  const recon_pose* src_poses, const recon_mvs_config* cfg,
                                                  int32_t* out_job) {
  return guard([&] {
    if (!ctx || !src_images || !ref_pose || !src_poses || !out_job) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    if (num_src < 1) fail(RECON_ERR_INVALID_ARGUMENT, "no source views");
    Context& C = *static_cast<Context*>(ctx);
    auto find = [&](int id) {
      auto it = C.images.find(id);
      if (it == C.images.end()) fail(RECON_ERR_INVALID_ARGUMENT, "unknown image id");
      return it->second;
    };
    std::vector<std::shared_ptr<StagedImage>> srcs;
    std::vector<recon_pose> poses(src_poses, src_poses + num_src);
    for (int k = 0; k < num_src; ++k) {
      if (src_images[k] == ref_image) fail(RECON_ERR_INVALID_ARGUMENT, "the reference is listed as a source");
      srcs.push_back(find(src_images[k]));
    }
    *out_job = build_job(C, find(ref_image), srcs, *ref_pose, poses, cfg, nullptr, 0);
  });
}

RECON_API recon_status recon_mvs_job_run(void* ctx, int32_t job) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    Context& C = *static_cast<Context*>(ctx);
    run_job(C, job);
  });
}

RECON_API recon_status recon_mvs_jobs_run(void* ctx, const int32_t* jobs, int32_t n) {
  return guard([&] {
    if (!ctx || (!jobs && n > 0)) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    Context& C = *static_cast<Context*>(ctx);
    run_jobs(C, std::vector<int>(jobs, jobs + n));
  });
}

// ---- the MVS stage over a whole capture ------------------------------------
// Orchestrator::StageMvs (orchestrator.cpp:942-1071) restated for the batched
// engine: every keyframe image staged once; per keyframe the sources of
// SelectSourceViews without itself and without image-less frames, at most
// num_views; the maps run in batches with the cancel check before each batch
// and a progress report after it; maps with nothing filled are dropped; the
// rest are fused (optionally behind the geometric-consistency filter) on the
// device.
}  // extern "C"

// The stage up to its fusion: staging, source selection, batched runs,
// consistency; then `fuse(maps)` with the produced maps (device pointers of
// jobs that live until it returns).
template <class Fuse>
static void stage_core(void* ctx, const uint8_t* const* gray, const int32_t* width, const int32_t* height,
                       const recon_pose* poses, const recon_camera_intrinsics* intr, int32_t num_keyframes,
                       const recon_mvs_config* cfg, const recon_mvs_stage_params* params, int32_t* out_maps,
                       Fuse&& fuse) {
    if (!ctx || !gray || !width || !height || !poses || !intr || !cfg)
      fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    if (out_maps) *out_maps = 0;
    recon_mvs_stage_params P;
    std::memset(&P, 0, sizeof(P));
    if (params) P = *params;
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    if (num_keyframes < 2) fail(RECON_ERR_MVS_NO_DEPTH, "fewer than two keyframes");
    const int N = num_keyframes;
    std::vector<std::shared_ptr<StagedImage>> img(N);
    for (int r = 0; r < N; ++r)
      if (gray[r]) img[r] = stage_image(C, gray[r], width[r], height[r], intr[r], P.undistort != 0);

    struct Jobs {  // every job of the stage is released on the way out
      Context& C;
      std::vector<int> ids;
      ~Jobs() {
        for (int id : ids) erase_job(C, id);
      }
    } jobs{C, {}};
    std::vector<int> ref_of;  // keyframe of each job
    std::vector<int32_t> sel(N);
    for (int r = 0; r < N; ++r) {
      if (!img[r]) continue;
      int32_t cnt = 0;
      const recon_status st = recon_mvs_select_source_views(&poses[r], poses, N, &intr[r], cfg, sel.data(), N, &cnt);
      if (st != RECON_OK) fail(st, "source view selection failed");
      std::vector<int> kept;
      for (int k = 0; k < cnt; ++k) {
        const int si = sel[k];
        if (si == r || si < 0 || si >= N || !img[si]) continue;
        kept.push_back(si);
      }
      if ((int)kept.size() > cfg->num_views) kept.resize(std::max(0, cfg->num_views));
      if (kept.empty()) continue;
      std::vector<std::shared_ptr<StagedImage>> srcs;
      std::vector<recon_pose> sp;
      for (int si : kept) {
        srcs.push_back(img[si]);
        sp.push_back(poses[si]);
      }
      jobs.ids.push_back(build_job(C, img[r], srcs, poses[r], sp, cfg, nullptr, 0));
      ref_of.push_back(r);
    }
    const int nj = (int)jobs.ids.size();
    const int batch = P.batch_size > 0 ? P.batch_size : std::max(1, nj);
    const bool compat = C.opts.mode != RECON_MVS_MODE_PLANE;
    DevArray<unsigned int> refined;
    refined.alloc(1);
    std::vector<unsigned int> filled(nj, 0);
    for (int start = 0; start < nj; start += batch) {
      if (P.cancel && P.cancel(P.user)) fail(RECON_ERR_CANCELLED, "cancelled");
      const int end = std::min(nj, start + batch);
      run_jobs(C, std::vector<int>(jobs.ids.begin() + start, jobs.ids.begin() + end));
      for (int j = start; j < end; ++j) {
        JobData& D = get_job(C, jobs.ids[j]);
        if (D.degenerate) continue;
        if (compat)  // PatchMatchStereo is followed by RefineSubpixel (orchestrator.cpp:1041-1044)
          CK(launch_compat_refine(D.J, D.out_depth.p, D.out_conf.p, D.inv_per_px, cfg->subpixel_fit_points,
                                  cfg->subpixel_iterations, refined.p, nullptr, nullptr, C.stream));
        CK(cudaMemcpyAsync(&filled[j], D.filled.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, C.stream));
      }
      CK(cudaStreamSynchronize(C.stream));
      if (P.progress) P.progress(P.user, (double)end / (double)nj);
    }
    std::vector<int> produced;
    for (int j = 0; j < nj; ++j)
      if (filled[j] > 0 && !get_job(C, jobs.ids[j]).degenerate) produced.push_back(j);
    if (produced.empty()) fail(RECON_ERR_MVS_NO_DEPTH, "no depth map produced");

    std::vector<std::unique_ptr<DevArray<uint8_t>>> keep(produced.size());
    if (P.consistency_views > 0) {
      std::vector<DevMap> dm;
      for (int j : produced) {
        const JobData& D = get_job(C, jobs.ids[j]);
        dm.push_back(DevMap{D.w, D.h, D.out_depth.p, img[ref_of[j]]->intr, poses[ref_of[j]]});
      }
      DevArray<uint8_t> count;
      for (size_t i = 0; i < produced.size(); ++i) {
        std::vector<DevMap> others;
        for (size_t q = 0; q < produced.size(); ++q)
          if (q != i) others.push_back(dm[q]);
        const size_t n = (size_t)dm[i].w * dm[i].h;
        count.alloc(n);
        keep[i] = std::make_unique<DevArray<uint8_t>>();
        keep[i]->alloc(n);
        consistency_device(C, dm[i], others, P.consistency_rel_depth, P.consistency_reproj_px, P.consistency_views,
                           count.p, keep[i]->p);
      }
    }
    std::vector<FuseMap> fm;
    for (size_t i = 0; i < produced.size(); ++i) {
      const JobData& D = get_job(C, jobs.ids[produced[i]]);
      const int r = ref_of[produced[i]];
      const float* nrm = (P.plane_normals && !compat) ? D.out_normal.p : nullptr;
      fm.push_back(fuse_map(D.w, D.h, D.out_depth.p, D.out_support.p, D.out_conf.p, keep[i] ? keep[i]->p : nullptr,
                            img[r]->intr, poses[r], nrm));
    }
    fuse(C, fm);
    if (out_maps) *out_maps = (int32_t)produced.size();
}

extern "C" {

RECON_API recon_status recon_mvs_stage_run(void* ctx, const uint8_t* const* gray, const int32_t* width,
                                           const int32_t* height, const recon_pose* poses,
                                           const recon_camera_intrinsics* intr, int32_t num_keyframes,
                                           const recon_mvs_config* cfg, const recon_mvs_stage_params* params,
                                           recon_mvs_point_cloud* out_cloud, int32_t* out_maps) {
  return guard([&] {
    if (!out_cloud) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out_cloud, 0, sizeof(*out_cloud));
    stage_core(ctx, gray, width, height, poses, intr, num_keyframes, cfg, params, out_maps,
               [&](Context& C, const std::vector<FuseMap>& fm) { fuse_maps(C, fm, *cfg, out_cloud); });
  });
}

// ---------------------------------------------------------------------------
// device-resident clouds
// ---------------------------------------------------------------------------
struct DeviceCloudImpl {
  int device = 0;
  DevCloud c;
  DevArray<float> colors, weights;
};

static void free_device_cloud(recon_mvs_device_cloud* out) {
  if (!out) return;
  auto* impl = static_cast<DeviceCloudImpl*>(out->impl);
  if (impl) {
    cudaSetDevice(impl->device);  // the arrays belong to that device
    delete impl;
  }
  std::memset(out, 0, sizeof(*out));
}

// Fills `out` from a device fusion result: the voxel records, zero colours
// (FuseDepthMaps writes none), the Poisson point weights max(0, confidence)
// (UnifiedPointCloud::ToOrientedCloud, orchestrator.cpp:181-193) and the
// bounds of the positions (PointCloudBounds without padding,
// orchestrator.cpp:80-99).
static void publish_device_cloud(Context& C, std::unique_ptr<DeviceCloudImpl> impl, recon_mvs_device_cloud* out) {
  const unsigned int n = impl->c.n;
  double bounds[6] = {1e30, 1e30, 1e30, -1e30, -1e30, -1e30};
  if (n > 0) {
    impl->colors.alloc(3 * (size_t)n);
    impl->weights.alloc(n);
    CK(cudaMemsetAsync(impl->colors.p, 0, 3 * sizeof(float) * (size_t)n, C.stream));
    DevArray<double> b;
    b.alloc(6);
    CK(launch_cloud_finish(impl->c.pos.p, impl->c.conf.p, n, impl->weights.p, b.p, C.stream));
    CK(cudaMemcpyAsync(bounds, b.p, sizeof(bounds), cudaMemcpyDeviceToHost, C.stream));
    CK(cudaStreamSynchronize(C.stream));
  }
  std::memset(out, 0, sizeof(*out));
  out->count = n;
  out->positions = impl->c.pos.p;
  out->normals = impl->c.nrm.p;
  out->colors = impl->colors.p;
  out->confidences = impl->c.conf.p;
  out->weights = impl->weights.p;
  out->keys = reinterpret_cast<int64_t*>(impl->c.key.p);
  out->counts = impl->c.cnt.p;
  for (int i = 0; i < 3; ++i) {
    out->bounds_lo[i] = bounds[i];
    out->bounds_hi[i] = bounds[3 + i];
  }
  out->device = C.device;
  impl->device = C.device;
  out->impl = impl.release();
}

RECON_API recon_status recon_mvs_stage_run_device(void* ctx, const uint8_t* const* gray, const int32_t* width,
                                                  const int32_t* height, const recon_pose* poses,
                                                  const recon_camera_intrinsics* intr, int32_t num_keyframes,
                                                  const recon_mvs_config* cfg, const recon_mvs_stage_params* params,
                                                  recon_mvs_device_cloud* out_cloud, int32_t* out_maps) {
  return guard([&] {
    if (!out_cloud) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out_cloud, 0, sizeof(*out_cloud));
    stage_core(ctx, gray, width, height, poses, intr, num_keyframes, cfg, params, out_maps,
               [&](Context& C, const std::vector<FuseMap>& fm) {
                 auto impl = std::make_unique<DeviceCloudImpl>();
                 fuse_maps_device(C, fm, *cfg, &impl->c);
                 publish_device_cloud(C, std::move(impl), out_cloud);
               });
  });
}

RECON_API recon_status recon_mvs_device_cloud_download(void* ctx, const recon_mvs_device_cloud* cloud,
                                                       recon_mvs_point_cloud* out) {
  return guard([&] {
    if (!ctx || !cloud || !out) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    const auto* impl = static_cast<const DeviceCloudImpl*>(cloud->impl);
    if (!impl && cloud->count > 0) fail(RECON_ERR_INVALID_ARGUMENT, "not a library device cloud");
    if (!impl) return;
    Context& C = *static_cast<Context*>(ctx);
    if (impl->device != C.device) fail(RECON_ERR_INVALID_ARGUMENT, "the cloud lives on another device");
    C.use();
    download_cloud(C, impl->c, out);
  });
}

RECON_API void recon_mvs_device_cloud_free(recon_mvs_device_cloud* cloud) { free_device_cloud(cloud); }

RECON_API recon_status recon_mvs_job_download(void* ctx, int32_t job, recon_mvs_depth_map* out, uint32_t* filled) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    download_job(C, get_job(C, job), out, filled);
  });
}

RECON_API recon_status recon_mvs_test_inject_tma_timeout(void* ctx) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    static_cast<Context*>(ctx)->test_tma_timeout = true;
  });
}

RECON_API recon_status recon_mvs_job_release(void* ctx, int32_t job) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    CK(cudaStreamSynchronize(C.stream));
    get_job(C, job);
    erase_job(C, job);
  });
}

RECON_API recon_status recon_mvs_synchronize(void* ctx) {
  return guard([&] {
    if (!ctx) fail(RECON_ERR_INVALID_ARGUMENT, "NULL context");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    CK(cudaStreamSynchronize(C.stream));
    finish_stats(C);
  });
}

RECON_API recon_status recon_mvs_context_stats(void* ctx, recon_mvs_stats* out) {
  return guard([&] {
    if (!ctx || !out) fail(RECON_ERR_INVALID_ARGUMENT, "NULL argument");
    Context& C = *static_cast<Context*>(ctx);
    C.use();
    read_counters(C);
    *out = C.stats;
  });
}

}  // extern "C"
