// bias.cu -- biases on the CV of every frame, on the device, so that a
// forward -> bias -> backward step never leaves the GPU.
//
//   hills      sum of truncated Gaussian hills of a one-dimensional CV, the
//              non-multivariate branch of MetaD::evaluateGaussian /
//              evaluateGaussianAndDerivatives (bias/MetaD.cpp:2148-2181,
//              2256-2273): dp = (s - c)/sigma, dp2 = dp^2/2, and for
//              dp2 < dp2cutoff = 6.25 (tools/Tools.h:71-74)
//                V += h*(A*exp(-dp2) + B),  dV/ds -= A*h*exp(-dp2)*dp/sigma
//              with A = 1/(1-exp(-6.25)), B = -exp(-6.25)/(1-exp(-6.25)) when
//              stretched, A = 1, B = 0 otherwise
//   restraint  Restraint::calculate (bias/Restraint.cpp:125-141):
//              V = kappa/2 (s-at)^2 + slope (s-at), dV/ds = kappa (s-at) + slope
//
// One block per frame for the hills; each thread sums a strided subset of the
// hills, and the block combines the partial sums in a fixed tree, so results
// do not depend on timing.
#include "coordgpu.h"
#include "launch.h"

#include <cmath>

namespace coordgpu {
namespace {

constexpr double kDp2Cutoff = 6.25;

__global__ void __launch_bounds__(256) k_bias_hills(int n_hills, const double *__restrict__ s,
                                                    const double *__restrict__ centers,
                                                    const double *__restrict__ sigmas,
                                                    const double *__restrict__ heights, double stretch_a,
                                                    double stretch_b, int accumulate, double *V, double *dVds) {
  const int f = blockIdx.x;
  const double sv = s[f];
  const double *c = centers + (size_t)f * n_hills;
  const double *sg = sigmas + (size_t)f * n_hills;
  const double *h = heights + (size_t)f * n_hills;
  double v = 0.0, d = 0.0;
  for (int i = threadIdx.x; i < n_hills; i += blockDim.x) {
    const double inv = 1.0 / sg[i];
    const double dp = (sv - c[i]) * inv;
    const double dp2 = 0.5 * dp * dp;
    if (dp2 < kDp2Cutoff) {
      const double e = h[i] * exp(-dp2);
      v += stretch_a * e + h[i] * stretch_b;
      d -= stretch_a * e * dp * inv;
    }
  }
  __shared__ double rv[256], rd[256];
  rv[threadIdx.x] = v;
  rd[threadIdx.x] = d;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      rv[threadIdx.x] += rv[threadIdx.x + o];
      rd[threadIdx.x] += rd[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (V) V[f] = accumulate ? V[f] + rv[0] : rv[0];
    if (dVds) dVds[f] = accumulate ? dVds[f] + rd[0] : rd[0];
  }
}

__global__ void k_bias_restraint(int n_frames, const double *__restrict__ s, double at, double kappa, double slope,
                                 int accumulate, double *V, double *dVds) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n_frames) return;
  const double cv = s[f] - at;
  const double e = 0.5 * kappa * cv * cv + slope * cv;
  const double g = kappa * cv + slope;
  if (V) V[f] = accumulate ? V[f] + e : e;
  if (dVds) dVds[f] = accumulate ? dVds[f] + g : g;
}

} // namespace
} // namespace coordgpu

using namespace coordgpu;

extern "C" {

int coord_bias_hills(int n_frames, const double *s, int n_hills, const double *centers, const double *sigmas,
                     const double *heights, int stretch, int accumulate, double *V, double *dVds, void *stream) {
  if (n_frames < 0 || n_hills < 0) return COORD_ERR_ARG;
  if (n_frames == 0) return COORD_OK;
  if (!s || (n_hills > 0 && (!centers || !sigmas || !heights))) return COORD_ERR_ARG;
  const double a = stretch ? 1.0 / (1.0 - std::exp(-kDp2Cutoff)) : 1.0;
  const double b = stretch ? -std::exp(-kDp2Cutoff) / (1.0 - std::exp(-kDp2Cutoff)) : 0.0;
  k_bias_hills<<<n_frames, 256, 0, (cudaStream_t)stream>>>(n_hills, s, centers, sigmas, heights, a, b, accumulate,
                                                            V, dVds);
  g_launches += 1;
  return cudaGetLastError() == cudaSuccess ? COORD_OK : COORD_ERR_CUDA;
}

int coord_bias_restraint(int n_frames, const double *s, double at, double kappa, double slope, int accumulate,
                         double *V, double *dVds, void *stream) {
  if (n_frames < 0) return COORD_ERR_ARG;
  if (n_frames == 0) return COORD_OK;
  if (!s) return COORD_ERR_ARG;
  k_bias_restraint<<<(n_frames + 127) / 128, 128, 0, (cudaStream_t)stream>>>(n_frames, s, at, kappa, slope,
                                                                             accumulate, V, dVds);
  g_launches += 1;
  return cudaGetLastError() == cudaSuccess ? COORD_OK : COORD_ERR_CUDA;
}

} // extern "C"
