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
//    in NewtonGaussian.py:74), one group of lanes per atom, then the reference's parameter update with its
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

// Change of the cell's KL term f log(f/g) - f + g when g = g0 (model +
// background) moves by d: d - f log1p(d/g0), written as
//   d (g0 - f)/g0 + f (t - log1p t),  t = d / g0,
// so that neither the new model value g0 + d (which would round d to the
// spacing of g0) nor a difference of two nearly equal terms is formed.
__device__ __forceinline__ double kl_cell_change(float f, float g0, float d) {
  if (!(f > 0.f)) return (double)d;
  const float t = d / g0;
  double phi;
  if (fabsf(t) < 0.0625f) {
    // t - log1p(t) = t^2/2 - t^3/3 + t^4/4 - ...  (|t| < 1/16: 8 terms)
    const double td = (double)t;
    double s2 = 1.0 / 9.0;
#pragma unroll
    for (int k = 8; k >= 2; --k) s2 = fma(s2, -td, 1.0 / (double)k);
    phi = td * td * s2;
  } else {
    phi = (double)t - log1p((double)t);
  }
  return (double)d * (double)((g0 - f) / g0) + (double)f * phi;
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
          acc += kl_cell_change(fo, Rv + u.bg, d);
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
// The blocks are assembled and solved in FP64.  On this GPU a dependent FP64
// operation takes about 64 cycles and an FP64 warp instruction holds the
// SM's FP64 pipe for 16 cycles, so a P x P factorisation run by one thread is
// one long dependent chain (about a thousand FP64 operations for P = 10, with
// divisions and square roots; 94 us for one block of 64 atoms).  Here a group
// of G >= P lanes shares one atom: lane l holds row l of the damped block,
// columns are broadcast with shuffles, each column costs one reciprocal
// square root (Cholesky) or one reciprocal (LU), after which the lanes update
// their rows independently; the dependent chain per column is a broadcast,
// the reciprocal and two multiply-adds.  A warp holds 32 / G groups: since
// an FP64 warp instruction costs the pipe the same whatever lanes it uses,
// G = P packs the most atoms into each (P = 10: three atoms a warp instead of
// two with G = 16), the last 32 mod G lanes idle.
//
// gshfl: lane k of the caller's group (base: its first lane); a power-of-two
// G uses the width-G shuffle, any other an explicit source lane.
template <int G, typename T>
__device__ __forceinline__ T gshfl(T v, int base, int k) {
  if constexpr ((G & (G - 1)) == 0) return __shfl_sync(0xffffffffu, v, k, G);
  else return __shfl_sync(0xffffffffu, v, base + k);
}
//
// Every lane of a warp executes every shuffle (no lane leaves early), so a
// group whose atom is out of range or masked runs on an identity block and
// stores nothing.

// Right-looking Cholesky H = L L^T on the group, then L y = b, L^T x = y.
// Lane l: a[] row l of the block (overwritten by row l of L), b = rhs[l].
// Returns (identically on all lanes of the group) whether every pivot was
// positive; x[] receives the solution on every lane.
template <int P, int G>
__device__ __forceinline__ bool group_cholesky(double (&a)[P], double b, int l, int base,
                                               double (&x)[P]) {
  double inv[P], col[P];
  bool spd = true;
#pragma unroll
  for (int k = 0; k < P; ++k) col[k] = 0.0;
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const double piv = gshfl<G>(a[j], base, j);
    spd = spd && (piv > 0.0);
    const double ij = rsqrt(piv > 0.0 ? piv : 1.0);
    inv[j] = ij;
    const double lij = (l == j) ? piv * ij : a[j] * ij;   // L[l][j] for l >= j
    a[j] = lij;
#pragma unroll
    for (int k = j + 1; k < P; ++k) {
      const double lkj = gshfl<G>(lij, base, k);
      if (l == j) col[k] = lkj;         // lane j keeps column j of L
      a[k] = fma(-lij, lkj, a[k]);      // trailing rows (only k <= l is used)
    }
  }
  // forward: y_j = (b_j - sum_{k<j} L[j][k] y_k) / L[j][j]; lane l folds
  // each y_j into its own b as soon as it is known
  double y[P];
#pragma unroll
  for (int j = 0; j < P; ++j) {
    y[j] = gshfl<G>(b, base, j) * inv[j];
    b = fma(-a[j], y[j], b);
  }
  // backward: x_i = (y_i - sum_{k>i} L[k][i] x_k) / L[i][i]; lane i holds
  // column i of L below the diagonal in col[]
  double acc = 0.0;
#pragma unroll
  for (int k = P - 1; k >= 0; --k) {
    const double v = (y[k] - acc) * inv[k];
    x[k] = gshfl<G>(v, base, k);
    acc = fma(col[k], x[k], acc);
  }
  return spd;
}

// Partial-pivoting LU (Gaussian elimination, as numpy.linalg.solve's LAPACK
// getrf/getrs) on the group, without moving rows: the pivot of column c is
// the largest |a[c]| among the rows not yet used as pivots (ties to the
// lower row), its row is broadcast and every other unused row eliminates
// column c with the multiplier a[c] * (1 / pivot).  Returns false for a
// zero pivot column.
template <int P, int G>
__device__ __forceinline__ bool group_lu(double (&a)[P], double b, int l, int base,
                                         double (&x)[P]) {
  constexpr unsigned kAll = 0xffffffffu;
  bool used = l >= P;                   // padding lanes never pivot
  bool ok = true;
  int prow[P];
  double pinv[P];
#pragma unroll
  for (int c = 0; c < P; ++c) {
    double v = used ? -1.0 : fabs(a[c]);
    int idx = l;
    if constexpr ((G & (G - 1)) == 0) {
#pragma unroll
      for (int off = G / 2; off > 0; off >>= 1) {
        const double ov = __shfl_xor_sync(kAll, v, off, G);
        const int oi = __shfl_xor_sync(kAll, idx, off, G);
        if (ov > v || (ov == v && oi < idx)) {
          v = ov;
          idx = oi;
        }
      }
    } else {
      // the same choice (largest, ties to the lower row) by a scan
      const double mine = v;
      v = -2.0;
#pragma unroll
      for (int i = 0; i < G; ++i) {
        const double ov = gshfl<G>(mine, base, i);
        if (ov > v) {
          v = ov;
          idx = i;
        }
      }
    }
    ok = ok && (v > 0.0);
    const double piv = gshfl<G>(a[c], base, idx);
    const double pi = 1.0 / (piv != 0.0 ? piv : 1.0);
    prow[c] = idx;
    pinv[c] = pi;
    const bool elim = !used && l != idx;
    const double m = a[c] * pi;
#pragma unroll
    for (int k = c + 1; k < P; ++k) {
      const double pk = gshfl<G>(a[k], base, idx);
      if (elim) a[k] = fma(-m, pk, a[k]);
    }
    const double pb = gshfl<G>(b, base, idx);
    if (elim) b = fma(-m, pb, b);
    used = used || l == idx;
  }
  // back substitution in pivot order: row prow[c] holds U[c][c..P-1]; every
  // lane folds each x_k into its rhs as soon as it is known
#pragma unroll
  for (int c = P - 1; c >= 0; --c) {
    x[c] = gshfl<G>(b * pinv[c], base, prow[c]);
    b = fma(-a[c], x[c], b);
  }
  return ok;
}

// theta (N, P) float64 in the derivative order [I, x, r]; writes theta_new
// and |dtheta|.  lam (N) adds lam_j to the diagonal.  mask (nullable): atoms
// with mask[j] == 0 keep their parameters.  One group of G lanes per atom;
// after the solve lane l forms parameter l only.
// The body of one 32-thread block (the launch's block; a multi-problem launch
// maps its blocks to (problem, block)).
template <int P, int D, int G>
__device__ __forceinline__ void solve_body(int n, const double *g, const double *H,
                                           const double *lam, const double *theta,
                                           const unsigned char *mask, double *theta_new,
                                           double *step_norm, int *fail, const AtomOut &ao,
                                           int block) {
  constexpr unsigned kAll = 0xffffffffu;
  constexpr int GPW = 32 / G;           // atoms per warp
  if (block * GPW >= n) return;         // whole warp past the last atom
  const int lane = (int)threadIdx.x & 31;
  const int grp = lane / G;             // GPW: the idle lanes past the last group
  const int l = lane - grp * G;
  const int base = grp * G;
  const int j = block * GPW + grp;
  const bool live = grp < GPW && j < n;
  const bool active = live && (mask == nullptr || mask[j] != 0);
  const bool row = live && l < P;
  double a[P], b, x[P];
  // the damped diagonal entry of row l, formed once
  const double diag = row ? H[((size_t)j * P + l) * P + l] + lam[j] : 1.0;
  auto load = [&]() {
#pragma unroll
    for (int k = 0; k < P; ++k)
      a[k] = k == l ? diag : (row ? H[((size_t)j * P + l) * P + k] : 0.0);
    b = row ? -g[(size_t)j * P + l] : 0.0;
  };
  load();
  bool ok = group_cholesky<P, G>(a, b, l, base, x);
  // some atom of this warp is not positive definite (idle lanes, which
  // shuffle other groups' values, do not count)
  if (__any_sync(kAll, live && !ok)) {
    const bool chol_ok = ok;
    load();
    double xl[P];
    const bool lu_ok = group_lu<P, G>(a, b, l, base, xl);
    if (!chol_ok) {
      ok = lu_ok;
#pragma unroll
      for (int k = 0; k < P; ++k) x[k] = xl[k];
    }
  }
#pragma unroll
  for (int k = 0; k < P; ++k)
    if (!(x[k] == x[k]) || fabs(x[k]) > 1e30) ok = false;
  ok = ok && active;
  // lane l: its step component and parameter
  double mine = 0.0;
#pragma unroll
  for (int k = 0; k < P; ++k)
    if (k == l) mine = x[k];
  const double d = (ok && row) ? mine : 0.0;
  double th = row ? theta[(size_t)j * P + l] : 0.0;
  th += d;
  // |dtheta| over the group, fixed butterfly order
  double nrm = d * d;
  if constexpr ((G & (G - 1)) == 0) {
#pragma unroll
    for (int off = 1; off < G; off <<= 1) nrm += __shfl_xor_sync(kAll, nrm, off, G);
  } else {
    const double mine = nrm;
    nrm = 0.0;
#pragma unroll
    for (int i = 0; i < G; ++i) nrm += gshfl<G>(mine, base, i);
  }
  // clamps of the reference's update: I >= 0, sign flips keeping
  // diag(r) >= 0 (P fixes the kind: 4 / 5 isotropic 2D / 3D, 6 anisotropic
  // 2D, 10 anisotropic 3D); a flip of r's diagonal entry i negates row i
  const unsigned neg = __ballot_sync(kAll, th < 0.0) >> base;
  if (ok) {
    const int q = l - 1 - D;             // index in packed r
    auto negr = [&](int i) { return ((neg >> (1 + D + i)) & 1u) != 0u; };
    if (l == 0 && th < 0.0) th = 0.0;
    if constexpr (P == 4 || P == 5) {
      if (q == 0) th = fabs(th);
    } else if constexpr (P == 6) {
      // packed [r00 r11 r01]: row 0 holds r00, r01
      if ((q == 0 || q == 2) && negr(0)) th = -th;
      if (q == 1 && negr(1)) th = -th;
    } else {
      // packed [r00 r11 r22 r01 r12 r02]: row 0 holds r00 r01 r02, row 1 r11 r12
      if ((q == 0 || q == 3 || q == 5) && negr(0)) th = -th;
      if ((q == 1 || q == 4) && negr(1)) th = -th;
      if (q == 2 && negr(2)) th = -th;
    }
  }
  if (!row) return;
  theta_new[(size_t)j * P + l] = th;
  if (l == 0) {
    step_norm[j] = sqrt(nrm);
    if (fail) fail[j] = (active && !ok) ? 1 : 0;
  }
  if (ao.I) {
    constexpr int PR = P - 1 - D;
    if (l == 0) ao.I[j] = (float)th;
    else if (l <= D) ao.x[(size_t)j * D + l - 1] = (float)th;
    else ao.r[(size_t)j * PR + l - 1 - D] = (float)th;
  }
}

template <int P, int D, int G>
__global__ void __launch_bounds__(32)
    gr_newton_solve_kernel(int n, const double *g, const double *H,
                           const double *lam, const double *theta,
                           const unsigned char *mask, double *theta_new,
                           double *step_norm, int *fail, AtomOut ao) {
  solve_body<P, D, G>(n, g, H, lam, theta, mask, theta_new, step_norm, fail, ao, blockIdx.x);
}

// dst[e] = src[e] for e in [0, n), the grid's threads striding from t0 by
// stride: float4 accesses when both arrays are 16-byte aligned, four of them
// loaded before any is stored, so a thread keeps 64 bytes in flight (a
// one-float copy loop keeps one float: the stores may alias the next loads).
__device__ __forceinline__ void copy_field(const float *__restrict__ src, float *__restrict__ dst,
                                           size_t n, size_t t0, size_t stride) {
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) != 0u) {
    for (size_t e = t0; e < n; e += stride) dst[e] = src[e];
    return;
  }
  const size_t n4 = n / 4;
  const float4 *s4 = reinterpret_cast<const float4 *>(src);
  float4 *d4 = reinterpret_cast<float4 *>(dst);
  size_t e = t0;
  for (; e + 3 * stride < n4; e += 4 * stride) {
    const float4 v0 = __ldcs(s4 + e), v1 = __ldcs(s4 + e + stride);
    const float4 v2 = __ldcs(s4 + e + 2 * stride), v3 = __ldcs(s4 + e + 3 * stride);
    d4[e] = v0;
    d4[e + stride] = v1;
    d4[e + 2 * stride] = v2;
    d4[e + 3 * stride] = v3;
  }
  for (; e < n4; e += stride) d4[e] = __ldcs(s4 + e);
  for (size_t i = 4 * n4 + t0; i < n; i += stride) dst[i] = src[i];
}

// Device-side accept/reject of a batched Newton trial (no host round trip):
// if loss_trial <= loss_cur the trial parameters (FP64 and the float32 atom
// arrays) become current, loss_cur takes the trial loss and the damping
// halves, else the damping grows tenfold (both clamped).  Appends
// (loss_cur, accepted) to the history.  Blocks stride over the atoms; each
// takes the decision itself.  Block 0 writes loss_cur last, and the decision
// does not change when another block reads loss_cur after that write (an
// accepted trial then compares equal; a rejected one leaves it untouched).
// The body of block `block` of `nblocks` 256-thread blocks (the launch's
// grid; a multi-problem launch maps its blocks to (problem, block)).
__device__ __forceinline__ void accept_body(int n, int P, int pr, int dim, double *loss_cur,
                                            const double *loss_trial, double *theta,
                                            const double *theta_trial, double *lam,
                                            double lam_min, double lam_max, const AtomOut &cur,
                                            const AtomIn &trial, double *hist, int *hist_acc,
                                            int *counter, int hist_len, const FieldCopy &fc,
                                            int block, int nblocks) {
  const bool acc = *loss_trial <= *loss_cur;
  const int stride = nblocks * 256;
  const int t0 = block * 256 + (int)threadIdx.x;
  if (acc)
    for (int e = t0; e < n * P; e += stride) theta[e] = theta_trial[e];
  for (int j = t0; j < n; j += stride) {
    double l = acc ? lam[j] * 0.5 : lam[j] * 10.0;
    lam[j] = l < lam_min ? lam_min : (l > lam_max ? lam_max : l);
    if (acc) {
      cur.I[j] = trial.I[j];
      for (int c = 0; c < dim; ++c) cur.x[(size_t)j * dim + c] = trial.x[(size_t)j * dim + c];
      for (int q = 0; q < pr; ++q) cur.r[(size_t)j * pr + q] = trial.r[(size_t)j * pr + q];
    }
  }
  // an accepted trial's fit fields become the current ones (so the next
  // iteration needs no projection of the current atoms)
  if (acc && fc.alpha) {
    copy_field(fc.alpha_t, fc.alpha, fc.n, t0, stride);
    if (fc.beta) copy_field(fc.beta_t, fc.beta, fc.n, t0, stride);
  }
  if (t0 == 0) {
    if (acc) *loss_cur = *loss_trial;
    const int k = *counter;
    if (k < hist_len) {
      hist[k] = *loss_cur;
      hist_acc[k] = acc ? 1 : 0;
    }
    *counter = k + 1;
  }
}

__global__ void __launch_bounds__(256)
    gr_newton_accept_kernel(int n, int P, int pr, int dim, double *loss_cur,
                            const double *loss_trial, double *theta,
                            const double *theta_trial, double *lam, double lam_min,
                            double lam_max, AtomOut cur, AtomIn trial, double *hist,
                            int *hist_acc, int *counter, int hist_len, FieldCopy fc) {
  accept_body(n, P, pr, dim, loss_cur, loss_trial, theta, theta_trial, lam, lam_min, lam_max,
              cur, trial, hist, hist_acc, counter, hist_len, fc, blockIdx.x, gridDim.x);
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
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  copy_field(alpha_t, alpha, n, t0, stride);
  if (beta) copy_field(beta_t, beta, n, t0, stride);
}

int launch_accept_fields(const double *loss_cur, const double *loss_trial, const float *alpha_t,
                         float *alpha, const float *beta_t, float *beta, size_t n,
                         cudaStream_t stream) {
  if (!loss_cur || !loss_trial || !alpha_t || !alpha || (beta && !beta_t)) return kErrArg;
  if (n == 0) return kOk;
  size_t blocks = (n / 4 + 255) / 256;       // a float4 per thread at least
  blocks = blocks < 1 ? 1 : (blocks > 152 * 16 ? 152 * 16 : blocks);
  gr_accept_fields_kernel<<<(unsigned)blocks, 256, 0, stream>>>(loss_cur, loss_trial, alpha_t,
                                                                alpha, beta_t, beta, n);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int launch_newton_accept(int n, int P, int pr, int dim, double *loss_cur,
                         const double *loss_trial, double *theta,
                         const double *theta_trial, double *lam, double lam_min,
                         double lam_max, AtomOut cur, AtomIn trial, double *hist,
                         int *hist_acc, int *counter, int hist_len, FieldCopy fc,
                         cudaStream_t stream) {
  if (fc.alpha && (!fc.alpha_t || (fc.beta && !fc.beta_t))) return kErrArg;
  const size_t work = (size_t)n * P > fc.n / 4 ? (size_t)n * P : fc.n / 4;
  size_t blocks = (work + 255) / 256;
  blocks = blocks < 1 ? 1 : (blocks > 152 * 8 ? 152 * 8 : blocks);
  gr_newton_accept_kernel<<<(unsigned)blocks, 256, 0, stream>>>(
      n, P, pr, dim, loss_cur, loss_trial, theta, theta_trial, lam, lam_min, lam_max, cur,
      trial, hist, hist_acc, counter, hist_len, fc);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int launch_newton_solve(int dim, int iso, int n, const double *g, const double *H,
                        const double *lam, const double *theta,
                        const unsigned char *mask, double *theta_new,
                        double *step_norm, int *fail, AtomOut ao, cudaStream_t stream) {
  if (n <= 0) return kOk;
  // one warp per block (32 / G atoms): the FP64 work then spreads over as
  // many SMs' FP64 pipes as there are warps
  auto blocks = [n](int G) { return (unsigned)((n + 32 / G - 1) / (32 / G)); };
  if (dim == 2 && iso)
    gr_newton_solve_kernel<4, 2, 4><<<blocks(4), 32, 0, stream>>>(n, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  else if (dim == 2)
    gr_newton_solve_kernel<6, 2, 6><<<blocks(6), 32, 0, stream>>>(n, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  else if (iso)
    gr_newton_solve_kernel<5, 3, 5><<<blocks(5), 32, 0, stream>>>(n, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  else
    gr_newton_solve_kernel<10, 3, 10><<<blocks(10), 32, 0, stream>>>(n, g, H, lam, theta, mask, theta_new, step_norm, fail, ao);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

// ---- multi-problem launches (2D) -------------------------------------------
template <int PP>
__global__ void __launch_bounds__(32)
    gr_batch_solve_kernel(const BatchProb *__restrict__ probs, const int *__restrict__ off, int n,
                          const int *__restrict__ active) {
  const int p = batch_find(off, n, blockIdx.x);
  if (!active[p]) return;
  const BatchProb &B = probs[p];
  const AtomOut ao{const_cast<float *>(B.trial.I), const_cast<float *>(B.trial.x),
                   const_cast<float *>(B.trial.r)};
  solve_body<PP, 2, 8>(B.cur.n, B.dout.g, B.dout.H, B.lam, B.theta, nullptr, B.theta_trial,
                       B.step, nullptr, ao, blockIdx.x - off[p]);
}

__global__ void __launch_bounds__(256)
    gr_batch_accept_kernel(const BatchProb *__restrict__ probs, const int *__restrict__ off,
                           int n, const int *__restrict__ active) {
  const int p = batch_find(off, n, blockIdx.x);
  if (!active[p]) return;
  const BatchProb &B = probs[p];
  const AtomOut cur{const_cast<float *>(B.cur.I), const_cast<float *>(B.cur.x),
                    const_cast<float *>(B.cur.r)};
  const AtomIn trial{B.trial.I, B.trial.x, B.trial.r};
  const FieldCopy none{nullptr, nullptr, nullptr, nullptr, 0};
  accept_body(B.cur.n, B.P, B.pr, 2, B.loss_cur, B.loss_trial, B.theta, B.theta_trial, B.lam,
              B.lam_min, B.lam_max, cur, trial, B.hist, B.hist_acc, B.counter, B.hist_len, none,
              blockIdx.x - off[p], off[p + 1] - off[p]);
}

int launch_batch_solve(const BatchLaunch &b, int P, cudaStream_t stream) {
  if (b.grid_solve <= 0) return kOk;
  if (P == 4)
    gr_batch_solve_kernel<4><<<b.grid_solve, 32, 0, stream>>>(b.probs, b.off_solve, b.n, b.active);
  else if (P == 6)
    gr_batch_solve_kernel<6><<<b.grid_solve, 32, 0, stream>>>(b.probs, b.off_solve, b.n, b.active);
  else
    return kErrArg;
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int launch_batch_accept(const BatchLaunch &b, cudaStream_t stream) {
  if (b.grid_acc <= 0) return kOk;
  gr_batch_accept_kernel<<<b.grid_acc, 256, 0, stream>>>(b.probs, b.off_acc, b.n, b.active);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int preload_update() {
  return preload_fn(gr_atom_update_kernel<1>) + preload_fn(gr_atom_update_kernel<2>) +
         preload_fn(gr_sum_partials_kernel) + preload_fn(gr_newton_solve_kernel<4, 2, 4>) +
         preload_fn(gr_newton_solve_kernel<6, 2, 6>) +
         preload_fn(gr_newton_solve_kernel<5, 3, 5>) +
         preload_fn(gr_newton_solve_kernel<10, 3, 10>) + preload_fn(gr_newton_accept_kernel) +
         preload_fn(gr_accept_fields_kernel) + preload_fn(gr_batch_solve_kernel<4>) +
         preload_fn(gr_batch_solve_kernel<6>) + preload_fn(gr_batch_accept_kernel);
}

}  // namespace gr
