// adjoint.cu -- the differentiation form: per-hypothesis gradients of the
// aggregated plane cost, and the pose normal equations for pose recovery.
// The math is in adjoint.cuh.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "adjoint.cuh"
#include "kernels.h"

namespace rmvs {

// Per hypothesis: cost, gradient (d, theta, phi), Gauss-Newton matrix (6)
// and, when pose_grad != nullptr, the gradient in every source's pose
// (num_src x 6).
template <int kMode>
__global__ void __launch_bounds__(128) k_plane_adjoint(Job J, int n, const int* __restrict__ px,
                                                       const int* __restrict__ py, const double* __restrict__ depth,
                                                       const double* __restrict__ angles, float* cost, float* grad,
                                                       float* gn, float* pose_grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  AdjHyp h;
  float c = kCostInf, g[3] = {0, 0, 0}, H[6] = {0, 0, 0, 0, 0, 0};
  float* pg = pose_grad ? pose_grad + (size_t)i * 6 * J.num_src : nullptr;
  if (make_adj_hyp(J, px[i], py[i], (float)depth[i], (float)angles[2 * i], (float)angles[2 * i + 1], &h)) {
    plane_adjoint<kMode>(J, h, &c, g, H, pg);
  } else if (pg) {
    for (int k = 0; k < 6 * J.num_src; ++k) pg[k] = 0.f;
  }
  cost[i] = c;
  for (int k = 0; k < 3; ++k) grad[3 * i + k] = g[k];
  if (gn)
    for (int k = 0; k < 6; ++k) gn[6 * i + k] = H[k];
}

// Pose normal equations: for every source s, over the given pixels (every
// view valid at a pixel counts, independent of best_k), the sums of the view
// cost c_s, its pose gradient (6) and Gauss-Newton matrix (21), and the
// number of contributing pixels.  One record of kPoseRec floats per (block,
// source); the host adds the blocks in order (deterministic).
constexpr int kPoseRec = 1 + 6 + kPoseH + 1;

template <int kMode>
__global__ void __launch_bounds__(128) k_pose_normal_eq(Job J, int n, const int* __restrict__ px,
                                                        const int* __restrict__ py, const double* __restrict__ depth,
                                                        const double* __restrict__ angles, float* partial) {
  __shared__ float red[4][kPoseRec];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  AdjHyp h;
  const bool ok = i < n && make_adj_hyp(J, px[i], py[i], (float)depth[i], (float)angles[2 * i],
                                        (float)angles[2 * i + 1], &h);
  for (int s = 0; s < J.num_src; ++s) {
    float rec[kPoseRec];
    for (int k = 0; k < kPoseRec; ++k) rec[k] = 0.f;
    if (ok) {
      const ViewGeo geo = view_geo(J, J.src[s], h);
      const ViewMom mo = view_moments<kMode>(J, J.src[s], geo, h);
      if (mo.valid) {
        float g[3], H[6];
        view_adjoint<kMode, true>(J, J.src[s], geo, h, mo, g, H, rec + 1, rec + 7);
        rec[0] = 1.0f - mo.ncc;
        rec[kPoseRec - 1] = 1.0f;
      }
    }
    // block sum: warp shuffles, then the 4 warps in order
    for (int k = 0; k < kPoseRec; ++k) {
      float v = rec[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kPoseRec) {
      const int k = threadIdx.x;
      partial[((size_t)blockIdx.x * J.num_src + s) * kPoseRec + k] =
          ((red[0][k] + red[1][k]) + red[2][k]) + red[3][k];
    }
    __syncthreads();
  }
}

template <class F>
static cudaError_t dispatch_mode(int mode, F&& f) {
  if (mode == kSrcBf16) return f(std::integral_constant<int, kSrcBf16>{});
  return f(std::integral_constant<int, kSrcExact>{});
}

cudaError_t launch_plane_adjoint(const Job& J, int n, const int* px, const int* py, const double* depth,
                                 const double* angles, float* cost, float* grad, float* gn, float* pose_grad,
                                 cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (J.num_src > kMaxSources) return cudaErrorInvalidValue;
  return dispatch_mode(J.src_mode, [&](auto m) {
    k_plane_adjoint<decltype(m)::value><<<(n + 127) / 128, 128, 0, st>>>(J, n, px, py, depth, angles, cost, grad,
                                                                          gn, pose_grad);
    return cudaGetLastError();
  });
}

int pose_partial_records() { return kPoseRec; }

cudaError_t launch_pose_normal_eq(const Job& J, int n, const int* px, const int* py, const double* depth,
                                  const double* angles, float* partial, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (J.num_src > kMaxSources) return cudaErrorInvalidValue;
  return dispatch_mode(J.src_mode, [&](auto m) {
    k_pose_normal_eq<decltype(m)::value><<<(n + 127) / 128, 128, 0, st>>>(J, n, px, py, depth, angles, partial);
    return cudaGetLastError();
  });
}

}  // namespace rmvs
