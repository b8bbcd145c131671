// Per-angle detector moments of a sinogram (sm_103a), for the moment-matching
// initial guess of a new atom.
//
// The reference's guess (KL_GaussRadon.py:57-121, doKL_ProjGDStep_iso) fits
// one Gaussian to the positive part of a residual sinogram from its moments:
// MOM0 (:227-229), MOM1 (:232-253) and MOM2 (:347-368), each a CPU loop over
// the sinogram.  Here one block per angle reads the target
//     f = max(0, res)                               (RR == NULL)
//     f = max(0, t res + (1 - t) scale RR)          (otherwise)
// cell by cell -- the blend of the reference's iteration, never stored -- and
// sums in FP64, in a fixed order,
//     S0[a] = sum f,  S1[a, i] = sum f p_i,  S2[a, i] = sum f p_i^2
// over its detector cells (p_i the cell coordinate along detector axis i).
// The spread about any centre follows on the host:
//     sum f (p_i - c)^2 = S2 - 2 c S1 + c^2 S0.
#include "gr_kernels.cuh"
#include "gauss_radon.h"

namespace gr {

constexpr int kMomThreads = 256;

template <int K>
__global__ void __launch_bounds__(kMomThreads)
    gr_moments_kernel(Geom g, const float *res, const float *rr, float t, float scale,
                      double *S0, double *S1, double *S2) {
  __shared__ double sh[kMomThreads][1 + 2 * K];
  const int a = blockIdx.x;
  const int D0 = g.ax[0].n, D1 = K == 2 ? g.ax[1].n : 1;
  const size_t cells = (size_t)D0 * D1;
  const size_t base = (size_t)a * cells;
  double s0 = 0.0, s1[K], s2[K];
#pragma unroll
  for (int i = 0; i < K; ++i) s1[i] = s2[i] = 0.0;
  for (size_t e = threadIdx.x; e < cells; e += kMomThreads) {
    float v = res[base + e];
    if (rr) v = t * v + (1.f - t) * scale * rr[base + e];
    if (!(v > 0.f)) continue;
    const double f = v;
    const int k0 = K == 2 ? (int)(e / D1) : (int)e;
    const double p0 = g.ax[0].coords[k0];
    s0 += f;
    s1[0] += f * p0;
    s2[0] += f * p0 * p0;
    if constexpr (K == 2) {
      const double p1 = g.ax[1].coords[e - (size_t)k0 * D1];
      s1[1] += f * p1;
      s2[1] += f * p1 * p1;
    }
  }
  sh[threadIdx.x][0] = s0;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    sh[threadIdx.x][1 + i] = s1[i];
    sh[threadIdx.x][1 + K + i] = s2[i];
  }
  __syncthreads();
  for (int o = kMomThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
#pragma unroll
      for (int q = 0; q < 1 + 2 * K; ++q) sh[threadIdx.x][q] += sh[threadIdx.x + o][q];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    S0[a] = sh[0][0];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      S1[(size_t)a * K + i] = sh[0][1 + i];
      S2[(size_t)a * K + i] = sh[0][1 + K + i];
    }
  }
}

int launch_moments(const Geom &g, const float *res, const float *rr, float t, float scale,
                   double *S0, double *S1, double *S2, cudaStream_t stream) {
  if (!res || !S0 || !S1 || !S2) return kErrArg;
  if (g.n_angles <= 0) return kOk;
  if (g.K == 1)
    gr_moments_kernel<1><<<g.n_angles, kMomThreads, 0, stream>>>(g, res, rr, t, scale, S0, S1, S2);
  else
    gr_moments_kernel<2><<<g.n_angles, kMomThreads, 0, stream>>>(g, res, rr, t, scale, S0, S1, S2);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int preload_moments() {
  return preload_fn(gr_moments_kernel<1>) + preload_fn(gr_moments_kernel<2>);
}

}  // namespace gr
