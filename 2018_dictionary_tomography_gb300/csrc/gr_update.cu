// Fitting-loop kernels (sm_103a).
//
// 1. gr_atom_update_kernel -- the per-atom step of the reference's fitting
//    loops (GD_lib._step, GD_lib.py:492-536): one atom moves from old to new
//    parameters; the sinogram changes by delta = R(new atom) - R(old atom)
//    only inside the union of the two support boxes.  In TRIAL mode the
//    kernel returns the exact change of the data fit (L2 or KL) without
//    writing anything; in APPLY mode it adds delta to the sinogram and
//    refreshes the fit's weight fields there.  The loop thus accepts or
//    rejects a step without re-projecting all atoms and without a restore:
//    a rejected trial leaves the state untouched, as the reference's
//    "R = R_old" does.  One warp per angle, lanes over the union box, each
//    cell handled by exactly one lane: deterministic.
// 2. gr_newton_solve_kernel -- batched damped Newton step for every atom:
//    (H_j + lambda_j 1) dtheta = -g_j in FP64 (Cholesky; partial-pivoting LU
//    when the damped block is not positive definite, like numpy.linalg.solve
//    in NewtonGaussian.py:74), then the reference's parameter update with its
//    clamps: I >= 0, and sign flips keeping diag(r) >= 0 (GD_lib.py:504-522).
#include "gr_kernels.cuh"

namespace gr {

struct UpdateArgs {
  int fit;            // kEpiL2 or kEpiKL
  int apply;          // 0: trial (read only), 1: apply
  float *R;           // sinogram
  const float *data;
  float bg;
  float *alpha;       // L2: R - data; KL: 1 - data/(R+b)
  float *beta;        // KL: data/(R+b)^2 (nullable)
  double *part;       // per-angle loss-change partials
};

__device__ __forceinline__ float kl_cell(float f, float g) {
  if (!(f > 0.f)) return g;
  const float e = (f - g) / g;
  float h;
  if (fabsf(e) < 0.125f) {
    const float e2 = e * e;
    h = e2 * (0.5f + e * (-1.f / 6.f + e * (1.f / 12.f + e * (-1.f / 20.f +
             e * (1.f / 30.f + e * (-1.f / 42.f + e * (1.f / 56.f)))))));
  } else {
    const float u = f / g;
    h = u * logf(u) - u + 1.f;
  }
  return g * h;
}

template <int K>
__device__ __forceinline__ float cell_value(const Pair<K> &p, bool ok, const Geom &g,
                                            int k0, int k1) {
  if (!ok || k0 < p.lo[0] || k0 > p.hi[0]) return 0.f;
  const float d0 = (g.ax[0].coords[k0] - p.qh[0]) - p.ql[0];
  float m;
  if constexpr (K == 2) {
    if (k1 < p.lo[1] || k1 > p.hi[1]) return 0.f;
    const float d1 = (g.ax[1].coords[k1] - p.qh[1]) - p.ql[1];
    m = fmaf(d0, fmaf(p.G[0], d0, 2.f * p.G[1] * d1), p.G[2] * d1 * d1);
  } else {
    m = p.G[0] * d0 * d0;
  }
  return m <= 1.f ? p.sgn * ex2_approx(fmaf(m, kNegThirtyLog2e, p.l2amp)) : 0.f;
}

template <int K>
__global__ void __launch_bounds__(128)
    gr_atom_update_kernel(Atoms olda, Atoms newa, Geom g, UpdateArgs u) {
  const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (a >= g.n_angles) return;
  Frame<K> f;
  load_frame<K>(g.frames, a, f);
  Pair<K> po, pn;
  const bool oko = pair_setup<K>(olda, 0, f, g, po) && po.lo[0] <= po.hi[0] &&
                   (K == 1 || po.lo[K - 1] <= po.hi[K - 1]);
  const bool okn = pair_setup<K>(newa, 0, f, g, pn) && pn.lo[0] <= pn.hi[0] &&
                   (K == 1 || pn.lo[K - 1] <= pn.hi[K - 1]);
  double acc = 0.0;
  if (oko || okn) {
    int lo[2] = {0, 0}, hi[2] = {0, 0};
#pragma unroll
    for (int k = 0; k < K; ++k) {
      lo[k] = oko ? (okn ? min(po.lo[k], pn.lo[k]) : po.lo[k]) : pn.lo[k];
      hi[k] = oko ? (okn ? max(po.hi[k], pn.hi[k]) : po.hi[k]) : pn.hi[k];
    }
    const int D0 = g.ax[0].n, D1 = K == 2 ? g.ax[1].n : 1;
    const int bw = hi[1] - lo[1] + 1;
    const int ncell = (hi[0] - lo[0] + 1) * bw;
    for (int e = lane; e < ncell; e += 32) {
      const int k0 = lo[0] + e / bw, k1 = lo[1] + e % bw;
      const float d = cell_value<K>(pn, okn, g, k0, k1) -
                      cell_value<K>(po, oko, g, k0, k1);
      if (d == 0.f) continue;
      const size_t gi = ((size_t)a * D0 + k0) * D1 + k1;
      const float Rv = u.R[gi];
      if (u.fit == kEpiL2) {
        const float res = u.alpha[gi];
        if (u.apply) {
          u.R[gi] = Rv + d;
          u.alpha[gi] = res + d;
        } else {
          acc += (double)d * ((double)res + 0.5 * (double)d);
        }
      } else {
        const float fo = u.data[gi];
        if (u.apply) {
          const float Rn = Rv + d;
          const float gg = Rn + u.bg, ig = 1.f / gg;
          u.R[gi] = Rn;
          u.alpha[gi] = 1.f - fo * ig;
          if (u.beta) u.beta[gi] = fo * ig * ig;
        } else {
          acc += (double)kl_cell(fo, Rv + d + u.bg) - (double)kl_cell(fo, Rv + u.bg);
        }
      }
    }
  }
  acc = warp_sum_d(acc);
  if (lane == 0 && u.part) u.part[a] = acc;
}

__global__ void gr_sum_partials_kernel(const double *part, int n, double *out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

int launch_atom_update(const Atoms &olda, const Atoms &newa, const Geom &g, int fit,
                       int apply, float *R, const float *data, float bg, float *alpha,
                       float *beta, double *dloss, void *ws, size_t ws_bytes,
                       cudaStream_t stream) {
  if (olda.n != 1 || newa.n != 1) return kErrArg;
  if (ws_bytes < align_up((size_t)g.n_angles * sizeof(double))) return kErrWorkspace;
  UpdateArgs u{fit, apply, R, data, bg, alpha, beta, static_cast<double *>(ws)};
  const int blocks = (g.n_angles * 32 + 127) / 128;
  if (g.K == 1) gr_atom_update_kernel<1><<<blocks, 128, 0, stream>>>(olda, newa, g, u);
  else gr_atom_update_kernel<2><<<blocks, 128, 0, stream>>>(olda, newa, g, u);
  note_launches(1);
  if (!apply && dloss) {
    gr_sum_partials_kernel<<<1, 256, 0, stream>>>(static_cast<double *>(ws), g.n_angles, dloss);
    note_launches(1);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

// ---------------------------------------------------------------------------
// batched damped Newton step
// ---------------------------------------------------------------------------
// Cholesky solve on the packed lower triangle L (row i holds entries
// i(i+1)/2 .. i(i+1)/2 + i), in place; every loop has a fixed trip count, so
// L and b stay in registers.  Returns false when the block is not positive
// definite (b is then unusable).
template <int P>
__device__ __forceinline__ bool cholesky_solve_packed(double (&L)[P * (P + 1) / 2],
                                                      double (&b)[P]) {
  bool spd = true;
#pragma unroll
  for (int i = 0; i < P; ++i) {
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      double s = L[i * (i + 1) / 2 + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= L[i * (i + 1) / 2 + k] * L[j * (j + 1) / 2 + k];
      if (i == j) {
        spd = spd && (s > 0.0);
        L[i * (i + 1) / 2 + i] = sqrt(s > 0.0 ? s : 1.0);
      } else {
        L[i * (i + 1) / 2 + j] = s / L[j * (j + 1) / 2 + j];
      }
    }
  }
  double y[P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    double s = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= L[i * (i + 1) / 2 + k] * y[k];
    y[i] = s / L[i * (i + 1) / 2 + i];
  }
#pragma unroll
  for (int i = P - 1; i >= 0; --i) {
    double s = y[i];
#pragma unroll
    for (int k = i + 1; k < P; ++k) s -= L[k * (k + 1) / 2 + i] * b[k];
    b[i] = s / L[i * (i + 1) / 2 + i];
  }
  return spd;
}

// partial-pivoting LU (Gaussian elimination) of a full block, in place
template <int P>
__device__ bool solve_lu(double (&A)[P][P], double (&b)[P]) {
  for (int c = 0; c < P; ++c) {
    int piv = c;
    double best = fabs(A[c][c]);
    for (int i = c + 1; i < P; ++i)
      if (fabs(A[i][c]) > best) {
        best = fabs(A[i][c]);
        piv = i;
      }
    if (best == 0.0) return false;
    if (piv != c) {
      for (int k = 0; k < P; ++k) {
        double t = A[c][k];
        A[c][k] = A[piv][k];
        A[piv][k] = t;
      }
      double t = b[c];
      b[c] = b[piv];
      b[piv] = t;
    }
    for (int i = c + 1; i < P; ++i) {
      const double m = A[i][c] / A[c][c];
      for (int k = c; k < P; ++k) A[i][k] -= m * A[c][k];
      b[i] -= m * b[c];
    }
  }
  for (int i = P - 1; i >= 0; --i) {
    double s = b[i];
    for (int k = i + 1; k < P; ++k) s -= A[i][k] * b[k];
    b[i] = s / A[i][i];
  }
  return true;
}

// theta (N, P) float64 in the derivative order [I, x, r]; writes theta_new
// and |dtheta|.  lam (N) adds lam_j to the diagonal.  mask (nullable): atoms
// with mask[j] == 0 keep their parameters.
template <int P, int D>
__global__ void gr_newton_solve_kernel(int n, int iso, const double *g, const double *H,
                                       const double *lam, const double *theta,
                                       const unsigned char *mask, double *theta_new,
                                       double *step_norm, int *fail, AtomOut ao) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  // Cholesky of the damped block (the common case) in registers; the full
  // block is re-read for the LU fallback only when it is not positive definite
  double L[P * (P + 1) / 2], b[P];
  const double lj = lam[j];
#pragma unroll
  for (int a = 0; a < P; ++a) {
    b[a] = -g[(size_t)j * P + a];
#pragma unroll
    for (int c = 0; c <= a; ++c)
      L[a * (a + 1) / 2 + c] = H[((size_t)j * P + a) * P + c] + (a == c ? lj : 0.0);
  }
  const bool active = mask == nullptr || mask[j] != 0;
  bool ok = false;
  if (active) {
    ok = cholesky_solve_packed<P>(L, b);
    if (!ok) {
      double A[P][P];
      for (int a = 0; a < P; ++a) {
        b[a] = -g[(size_t)j * P + a];
        for (int c = 0; c < P; ++c) A[a][c] = H[((size_t)j * P + a) * P + c];
        A[a][a] += lj;
      }
      ok = solve_lu<P>(A, b);
    }
  }
  for (int a = 0; a < P; ++a)
    if (!(b[a] == b[a]) || fabs(b[a]) > 1e30) ok = false;
  double nrm = 0.0;
  double t[P];
  for (int a = 0; a < P; ++a) {
    const double d = ok ? b[a] : 0.0;
    nrm += d * d;
    t[a] = theta[(size_t)j * P + a] + d;
  }
  if (ok) {
    t[0] = t[0] < 0.0 ? 0.0 : t[0];
    if (iso) {
      t[1 + D] = fabs(t[1 + D]);
    } else if (D == 2) {
      double *r = t + 1 + D;
      if (r[0] < 0) { r[0] = -r[0]; r[2] = -r[2]; }
      if (r[1] < 0) r[1] = -r[1];
    } else {
      double *r = t + 1 + D;
      if (r[0] < 0) { r[0] = -r[0]; r[3] = -r[3]; r[5] = -r[5]; }
      if (r[1] < 0) { r[1] = -r[1]; r[4] = -r[4]; }
      if (r[2] < 0) r[2] = -r[2];
    }
  } else {
    for (int a = 0; a < P; ++a) t[a] = theta[(size_t)j * P + a];
  }
  for (int a = 0; a < P; ++a) theta_new[(size_t)j * P + a] = t[a];
  step_norm[j] = sqrt(nrm);
  if (fail) fail[j] = (active && !ok) ? 1 : 0;
  if (ao.I) {
    constexpr int PR = P - 1 - D;
    ao.I[j] = (float)t[0];
    for (int c = 0; c < D; ++c) ao.x[(size_t)j * D + c] = (float)t[1 + c];
    for (int q = 0; q < PR; ++q) ao.r[(size_t)j * PR + q] = (float)t[1 + D + q];
  }
}

// Device-side accept/reject of a batched Newton trial (no host round trip):
// one block; if loss_trial <= loss_cur the trial parameters (FP64 and the
// float32 atom arrays) become current, loss_cur takes the trial loss and the
// damping halves, else the damping grows tenfold (both clamped).  Appends
// (loss_cur, accepted) to the history.
__global__ void gr_newton_accept_kernel(int n, int P, int pr, int dim,
                                        double *loss_cur, const double *loss_trial,
                                        double *theta, const double *theta_trial,
                                        double *lam, double lam_min, double lam_max,
                                        AtomOut cur, AtomIn trial, double *hist,
                                        int *hist_acc, int *counter, int hist_len) {
  __shared__ int acc;
  if (threadIdx.x == 0) acc = (*loss_trial <= *loss_cur) ? 1 : 0;
  __syncthreads();
  for (int e = threadIdx.x; e < n * P; e += blockDim.x)
    if (acc) theta[e] = theta_trial[e];
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double l = acc ? lam[j] * 0.5 : lam[j] * 10.0;
    lam[j] = l < lam_min ? lam_min : (l > lam_max ? lam_max : l);
    if (acc) {
      cur.I[j] = trial.I[j];
      for (int c = 0; c < dim; ++c) cur.x[(size_t)j * dim + c] = trial.x[(size_t)j * dim + c];
      for (int q = 0; q < pr; ++q) cur.r[(size_t)j * pr + q] = trial.r[(size_t)j * pr + q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (acc) *loss_cur = *loss_trial;
    const int k = *counter;
    if (k < hist_len) {
      hist[k] = *loss_cur;
      hist_acc[k] = acc;
    }
    *counter = k + 1;
  }
}

// After gr_newton_accept: when the trial was accepted (the accept kernel
// then set loss_cur to exactly loss_trial; a rejected trial has a larger
// loss), the trial's fit fields become the current ones, so the next
// iteration needs no projection of the current atoms.
__global__ void __launch_bounds__(256)
    gr_accept_fields_kernel(const double *loss_cur, const double *loss_trial,
                            const float *alpha_t, float *alpha, const float *beta_t,
                            float *beta, size_t n) {
  if (!(*loss_cur == *loss_trial)) return;  // rejected: keep the current fields
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    alpha[e] = alpha_t[e];
    if (beta) beta[e] = beta_t[e];
  }
}

int launch_accept_fields(const double *loss_cur, const double *loss_trial, const float *alpha_t,
                         float *alpha, const float *beta_t, float *beta, size_t n,
                         cudaStream_t stream) {
  if (!loss_cur || !loss_trial || !alpha_t || !alpha || (beta && !beta_t)) return kErrArg;
  if (n == 0) return kOk;
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  gr_accept_fields_kernel<<<(unsigned)blocks, 256, 0, stream>>>(loss_cur, loss_trial, alpha_t,
                                                                alpha, beta_t, beta, n);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int launch_newton_accept(int n, int P, int pr, int dim, double *loss_cur,
                         const double *loss_trial, double *theta,
                         const double *theta_trial, double *lam, double lam_min,
                         double lam_max, AtomOut cur, AtomIn trial, double *hist,
                         int *hist_acc, int *counter, int hist_len, cudaStream_t stream) {
  gr_newton_accept_kernel<<<1, 256, 0, stream>>>(n, P, pr, dim, loss_cur, loss_trial, theta,
                                                 theta_trial, lam, lam_min, lam_max, cur,
                                                 trial, hist, hist_acc, counter, hist_len);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int launch_newton_solve(int dim, int iso, int n, const double *g, const double *H,
                        const double *lam, const double *theta,
                        const unsigned char *mask, double *theta_new,
                        double *step_norm, int *fail, AtomOut ao, cudaStream_t stream) {
  if (n <= 0) return kOk;
  const int blocks = (n + 63) / 64;
  if (dim == 2 && iso)
    gr_newton_solve_kernel<4, 2><<<blocks, 64, 0, stream>>>(n, 1, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  else if (dim == 2)
    gr_newton_solve_kernel<6, 2><<<blocks, 64, 0, stream>>>(n, 0, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  else if (iso)
    gr_newton_solve_kernel<5, 3><<<blocks, 64, 0, stream>>>(n, 1, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  else
    gr_newton_solve_kernel<10, 3><<<blocks, 64, 0, stream>>>(n, 0, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

}  // namespace gr
