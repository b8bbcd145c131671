// Shared device helpers for the Gaussian-atom Radon kernels (sm_103a).
//
// Model (reference GaussDictCode/bin/NewtonBases2D.py:39-72 and
// GaussDictCode/bin/NewtonBases.py:262-310): an atom (I, x, r) projects to
//     R(y) = I / |r T| * exp(-30 m),   m = |(1 - t t^T) r (y - x)|^2,
//     t = r T / |r T|,   R = 0 where m > 1,
// for detector points y = sum_i q_i w_i.  With the frame B = [w_0 .. w_{K-1}, T]
// and K_c = r B_c, Q = K^T K, the projection of the atom is the Gaussian
//     m(q) = (q - q*)^T G (q - q*),  G = Q_ww - Q_wT Q_wT^T / Q_TT,
//     q* = (B^{-1} x)[0:K],          1/|r T| = Q_TT^{-1/2},
// i.e. a K-dimensional Gaussian whose precision is the Schur complement of
// the atom precision in the frame.  Per (atom, angle) "pair" the kernels
// compute G, q*, the amplitude and the support box once, and per detector
// cell only the quadratic form and one exp2.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gr {

constexpr int kMaxK = 2;                          // detector dimensions
constexpr float kNegThirtyLog2e = -43.28085122666891f;  // -30 / ln 2
constexpr int kFrameStride2D = 8;   // T(2) w0(2) wt0(2) wl0(2)
constexpr int kFrameStride3D = 24;  // T(3) w0(3) w1(3) wt0(3) wt1(3) wl0(3) wl1(3) pad(3)

// Error codes shared with the C ABI.
enum Status : int {
  kOk = 0,
  kErrArg = -1,
  kErrWorkspace = -2,
  kErrLaunch = -3,
  kErrShape = -4,
};

__device__ __forceinline__ float ex2_approx(float v) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(v));
  return y;
}

__device__ __forceinline__ float lg2_approx(float v) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(v));
  return y;
}

// Error-free transforms (Knuth TwoSum, FMA TwoProduct) used for the
// compensated projection centre and compensated accumulators.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Compensated dot product of length n <= 3 (Ogita-Rump-Oishi Dot2): the
// result hi + lo carries roughly twice the working precision.
template <int N>
__device__ __forceinline__ void dot2(const float *a, const float *b, float &hi,
                                     float &lo) {
  float s, c;
  two_prod(a[0], b[0], s, c);
#pragma unroll
  for (int i = 1; i < N; ++i) {
    float p, pe, t, te;
    two_prod(a[i], b[i], p, pe);
    two_sum(s, p, t, te);
    s = t;
    c += pe + te;
  }
  two_sum(s, c, hi, lo);
}

// Kahan-style compensated accumulator (Neumaier variant, exact when |v|>|s|).
struct CAcc {
  float s, c;
  __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float v) {
    float t = s + v;
    c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
    s = t;
  }
  __device__ __forceinline__ float get() const { return s + c; }
};

// Uniform detector grid: the coordinate of cell k is coords[k]; first and
// inverse step locate the support box, the stored coordinates are what the
// cell values use.
struct DetAxis {
  const float *coords;
  int n;
  float first;
  float inv_step;
};

// Geometry of one problem in device memory.
struct Geom {
  int K;                 // 1: 2D sinogram (A, D0); 2: 3D / 2.5D (A, D0, D1)
  int n_angles;
  const float *frames;   // n_angles x stride, see kFrameStride*
  DetAxis ax[kMaxK];
};

// Atoms in device memory: r is packed upper-triangular (2D: r00 r11 r01;
// 3D: r00 r11 r22 r01 r12 r02) or, when r_iso, one radius per atom.
struct Atoms {
  int n;
  const float *I;
  const float *x;
  const float *r;
  int r_iso;
  const int *order;  // optional processing order of the derivative kernels
};

template <int K>
struct Frame {
  float T[K + 1];
  float w[K][K + 1];
  float wt[K][K + 1];  // rows 0..K-1 of B^{-1} (rounded to FP32)
  const float *wl;     // their rounding residues (B^{-1} rows = wt + wl), read
                       // from the record only when a pair is set up
};

template <int K>
__device__ __forceinline__ void load_frame(const float *frames, int a,
                                           Frame<K> &f) {
  constexpr int D = K + 1;
  const float *p = frames + (size_t)a * (K == 1 ? kFrameStride2D : kFrameStride3D);
#pragma unroll
  for (int i = 0; i < D; ++i) f.T[i] = p[i];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int i = 0; i < D; ++i) f.w[k][i] = p[D * (1 + k) + i];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int i = 0; i < D; ++i) f.wt[k][i] = p[D * (1 + K + k) + i];
  f.wl = p + D * (1 + 2 * K);
}

// Upper-triangular r as a dense (K+1)x(K+1) matrix.
template <int K>
__device__ __forceinline__ void load_r(const Atoms &at, int j,
                                       float (&M)[K + 1][K + 1]) {
  constexpr int D = K + 1;
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) M[a][b] = 0.f;
  if (at.r_iso) {
    float s = at.r[j];
#pragma unroll
    for (int a = 0; a < D; ++a) M[a][a] = s;
  } else if constexpr (K == 1) {
    const float *r = at.r + 3 * (size_t)j;
    M[0][0] = r[0];
    M[1][1] = r[1];
    M[0][1] = r[2];
  } else {
    const float *r = at.r + 6 * (size_t)j;
    M[0][0] = r[0];
    M[1][1] = r[1];
    M[2][2] = r[2];
    M[0][1] = r[3];
    M[1][2] = r[4];
    M[0][2] = r[5];
  }
}

// Packed r index p -> (row, col).
template <int K>
__host__ __device__ constexpr int rrow(int p) {
  return K == 1 ? (p == 0 ? 0 : p == 1 ? 1 : 0)
                : (p == 0 ? 0 : p == 1 ? 1 : p == 2 ? 2 : p == 3 ? 0 : p == 4 ? 1 : 0);
}
template <int K>
__host__ __device__ constexpr int rcol(int p) {
  return K == 1 ? (p == 0 ? 0 : p == 1 ? 1 : 1)
                : (p == 0 ? 0 : p == 1 ? 1 : p == 2 ? 2 : p == 3 ? 1 : p == 4 ? 2 : 2);
}
template <int K>
__host__ __device__ constexpr int n_rparam() { return K == 1 ? 3 : 6; }

// Per (atom, angle) projection data.
template <int K>
struct Pair {
  float qh[K], ql[K];  // projection centre q* = hi + lo
  float G[3];          // G00, G01, G11 (K == 1: G00)
  float n;             // 1 / |r T|
  float l2amp;         // log2(|I| n)
  float sgn;           // sign of I (+1 or -1)
  int lo[K], hi[K];    // inclusive support box in cell indices (empty: lo > hi)
  // quantities kept for the derivative assembly
  float Kc[K + 1][K + 1];  // Kc[c][a] = (r B_c)_a, c = 0..K-1 detector axes, K = T
  float Q[K + 1][K + 1];   // Q[c][d] = Kc[c] . Kc[d]
};

template <int K>
__device__ __forceinline__ bool pair_setup(const Atoms &at, int j,
                                           const Frame<K> &f, const Geom &g,
                                           Pair<K> &p) {
  constexpr int D = K + 1;
  float M[D][D];
  load_r<K>(at, j, M);
  // K_c = r B_c for the detector axes and the ray direction
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const float *B = (c < K) ? f.w[c] : f.T;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      float s = 0.f;
#pragma unroll
      for (int b = a; b < D; ++b) s = fmaf(M[a][b], B[b], s);
      p.Kc[c][a] = s;
    }
  }
#pragma unroll
  for (int c = 0; c < D; ++c)
#pragma unroll
    for (int d = c; d < D; ++d) {
      float s = 0.f;
#pragma unroll
      for (int a = 0; a < D; ++a) s = fmaf(p.Kc[c][a], p.Kc[d][a], s);
      p.Q[c][d] = s;
      p.Q[d][c] = s;
    }
  const float qtt = p.Q[K][K];
  const float iqtt = 1.f / qtt;
  p.n = rsqrtf(qtt);
  // G = U^T U with U_i = K_i - t (t . K_i), t = K_T / |K_T| (the projected
  // detector axes); this Gram form stays positive semi-definite in FP32.
  float U[K][D];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const float c = p.Q[i][K] * iqtt;
#pragma unroll
    for (int a = 0; a < D; ++a) U[i][a] = fmaf(-c, p.Kc[K][a], p.Kc[i][a]);
  }
  if constexpr (K == 1) {
    p.G[0] = U[0][0] * U[0][0] + U[0][1] * U[0][1];
    p.G[1] = 0.f;
    p.G[2] = 0.f;
  } else {
    float g00 = 0.f, g01 = 0.f, g11 = 0.f;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      g00 = fmaf(U[0][a], U[0][a], g00);
      g01 = fmaf(U[0][a], U[1][a], g01);
      g11 = fmaf(U[1][a], U[1][a], g11);
    }
    p.G[0] = g00;
    p.G[1] = g01;
    p.G[2] = g11;
  }
  const float I = at.I[j];
  p.l2amp = lg2_approx(fabsf(I) * p.n);
  p.sgn = I < 0.f ? -1.f : 1.f;
  float xv[D];
#pragma unroll
  for (int a = 0; a < D; ++a) xv[a] = at.x[(size_t)D * j + a];
#pragma unroll
  // q* = (B^{-1} x)[k] with B^{-1} carried as wt + wl: a dual row rounded to
  // FP32 alone moves the centre by up to ~4e-8, which for the sharpest atoms
  // (r ~ 50) is a 2e-5 relative change of the basis at half its peak
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float hi, lo;
    dot2<D>(f.wt[k], xv, hi, lo);
#pragma unroll
    for (int a = 0; a < D; ++a) lo = fmaf(__ldg(f.wl + k * D + a), xv[a], lo);
    two_sum(hi, lo, p.qh[k], p.ql[k]);
  }

  // support box of m <= 1: |d_i| <= sqrt((G^{-1})_ii)
  float hw[K];
  bool ok;
  if constexpr (K == 1) {
    ok = p.G[0] > 0.f && qtt > 0.f;
    hw[0] = rsqrtf(p.G[0]);
  } else {
    float det = p.G[0] * p.G[2] - p.G[1] * p.G[1];
    ok = p.G[0] > 0.f && det > 0.f && qtt > 0.f;
    float idet = 1.f / det;
    hw[0] = sqrtf(p.G[2] * idet);
    hw[1] = sqrtf(p.G[0] * idet);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const DetAxis &ax = g.ax[k];
    // coordinates increase with the cell index (checked on the host)
    float c = (p.qh[k] - ax.first) * ax.inv_step;
    float h = hw[k] * ax.inv_step * 1.0001f + 1e-3f;
    float lo = ceilf(c - h), hi = floorf(c + h);
    bool fin = ok && (lo == lo) && (hi == hi) && fabsf(c) < 1e8f && h < 1e8f;
    p.lo[k] = fin ? max(0, (int)lo) : 1;
    p.hi[k] = fin ? min(ax.n - 1, (int)hi) : 0;
  }
  return ok;
}

// Squared Mahalanobis distance of cell offsets d from the centre.
template <int K>
__device__ __forceinline__ float quad(const Pair<K> &p, const float *d) {
  if constexpr (K == 1) return p.G[0] * d[0] * d[0];
  else return fmaf(d[0], fmaf(p.G[0], d[0], 2.f * p.G[1] * d[1]), p.G[2] * d[1] * d[1]);
}

// ---- pixel-integrated ("point spread") operator -------------------------
// Reference: GaussDictCode/bin/point_spread_functions.py.  A cell's value is
// the integral of the projection over the square cell of half-width s, by an
// 11-point (2D) or 11 x 11 (3D) rule over the cell clipped to the box
// +-rr around the atom centre, rr = 1 / min(diag r) (__Radius :24); the
// points sit at lo + t (hi - lo)/10, t = 1..11 (__rf2 :413, __rf3 :462) and
// the point values carry no m > 1 cut-off (__Rf :386).  A cell farther than
// rr + s from the centre is 0; an atom within s - rr of the cell centre gives
// the total mass I sqrt(pi/30)/(r00 r11) or I (pi/30)/(r00 r11 r22) (__total
// :60) with zero derivatives (__drf2 :924).  Distances are measured in the
// detector plane (orthonormal frames).
template <int K>
struct PsfPair {
  float rr, total;
  int lo[K], hi[K];  // cells that can be non-zero
};

template <int K>
__device__ __forceinline__ void psf_setup(const Atoms &at, int j, const Geom &g,
                                          const Pair<K> &p, bool ok, float s,
                                          PsfPair<K> &q) {
  constexpr int D = K + 1;
  float M[D][D];
  load_r<K>(at, j, M);
  float mn = fminf(M[0][0], M[1][1]);
  float prod = M[0][0] * M[1][1];
  if constexpr (K == 2) {
    mn = fminf(mn, M[2][2]);
    prod *= M[2][2];
  }
  q.rr = 1.f / mn;
  const float I = at.I[j];
  q.total = K == 1 ? I / prod * 0.32360019f : I / prod * 0.10471976f;  // sqrt(pi/30), pi/30
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const DetAxis &ax = g.ax[k];
    const float c = (p.qh[k] - ax.first) * ax.inv_step;
    const float h = (q.rr + s) * ax.inv_step + 1.001f;
    const float lo = ceilf(c - h), hi = floorf(c + h);
    const bool fin = ok && (lo == lo) && (hi == hi) && fabsf(c) < 1e8f && h < 1e8f;
    q.lo[k] = fin ? max(0, (int)lo) : 1;
    q.hi[k] = fin ? min(ax.n - 1, (int)hi) : 0;
  }
}

// Kind of a cell: 0 empty, 1 total, 2 quadrature; fills the quadrature
// start (offset from the atom centre) and step per axis.
template <int K>
__device__ __forceinline__ int psf_cell_kind(const PsfPair<K> &q, const float *dc,
                                             float s, float *base, float *step) {
  float n2 = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) n2 = fmaf(dc[k], dc[k], n2);
  const float n = sqrtf(n2);
  if (n + q.rr < s) return 1;
  if (n - q.rr > s) return 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const float c = -dc[k];  // atom centre relative to the cell centre
    const float lo = fmaxf(c - q.rr, -s), hi = fminf(c + q.rr, s);
    step[k] = 0.1f * (hi - lo);
    base[k] = dc[k] + lo;     // point offsets from the atom centre: base + t step
  }
  return 2;
}

// Pixel integral of E = n exp(-30 m) (times |I| through l2amp) over the
// quadrature points; returns the sum of point values times the rule's scale.
template <int K>
__device__ __forceinline__ float psf_quadrature(const Pair<K> &p, const float *base,
                                                const float *step) {
  float sum = 0.f;
  if constexpr (K == 1) {
#pragma unroll
    for (int t = 1; t <= 11; ++t) {
      const float d = fmaf((float)t, step[0], base[0]);
      sum += ex2_approx(fmaf(p.G[0] * d * d, kNegThirtyLog2e, p.l2amp));
    }
    return sum * (10.f * step[0] / 11.f);
  } else {
    for (int t = 1; t <= 11; ++t) {
      const float d0 = fmaf((float)t, step[0], base[0]);
      const float t0 = p.G[0] * d0 * d0, u = 2.f * p.G[1] * d0;
#pragma unroll
      for (int v = 1; v <= 11; ++v) {
        const float d1 = fmaf((float)v, step[1], base[1]);
        const float m = fmaf(d1, fmaf(p.G[2], d1, u), t0);
        sum += ex2_approx(fmaf(m, kNegThirtyLog2e, p.l2amp));
      }
    }
    return sum * (100.f * step[0] * step[1] / 121.f);
  }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Reduce-scatter of 32 values over the warp (recursive halving): on return
// v[0] of lane l is the sum over all lanes of their v[l].  At the step with
// offset m each lane keeps the half of its remaining values whose index bit m
// matches its lane bit and receives the partner's copy of that half.
__device__ __forceinline__ void warp_reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    const bool up = (lane & m) != 0;
#pragma unroll
    for (int k = 0; k < m; ++k) {
      const float keep = up ? v[k + m] : v[k];
      const float give = up ? v[k] : v[k + m];
      v[k] = keep + __shfl_xor_sync(0xffffffffu, give, m);
    }
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp sums n FP64 partials (written by other blocks before a
// __threadfence) in a fixed order and writes the total to *out.  A dependent
// FP64 add takes about 64 cycles on this GPU, so lane l keeps kSums running
// sums -- element i goes to sum (i / 32) % kSums of lane i % 32 -- and the
// dependent chain is n / (32 kSums) adds instead of n / 32; the sums are
// then combined pairwise and across the warp, always in the same order.
__device__ __forceinline__ void sum_partials_warp(const double *part, int n, double *out,
                                                  int lane) {
  constexpr int kSums = 8;
  double s[kSums];
#pragma unroll
  for (int k = 0; k < kSums; ++k) s[k] = 0.0;
  for (int base = 0; base < n; base += 32 * kSums) {
#pragma unroll
    for (int k = 0; k < kSums; ++k) {
      const int i = base + 32 * k + lane;
      if (i < n) s[k] += __ldcg(part + i);
    }
  }
#pragma unroll
  for (int w = 1; w < kSums; w <<= 1)
#pragma unroll
    for (int k = 0; k < kSums; k += 2 * w) s[k] += s[k + w];
  const double t = warp_sum_d(s[0]);
  if (lane == 0) *out = t;
}

// The same with all NW warps of a block (every thread calls it): thread k
// keeps 4 running sums over elements k + NW*32*(4 i + s); the threads' sums
// are combined pairwise, across each warp, then across the warps in order.
template <int NW>
__device__ __forceinline__ void sum_partials_block(const double *part, int n, double *out) {
  constexpr int T = NW * 32;
  constexpr int kSums = 4;
  __shared__ double ws[NW];
  const int tid = threadIdx.x;
  double s[kSums];
#pragma unroll
  for (int k = 0; k < kSums; ++k) s[k] = 0.0;
  for (int base = 0; base < n; base += T * kSums) {
#pragma unroll
    for (int k = 0; k < kSums; ++k) {
      const int i = base + T * k + tid;
      if (i < n) s[k] += __ldcg(part + i);
    }
  }
  s[0] += s[1];
  s[2] += s[3];
  const double t = warp_sum_d(s[0] + s[2]);
  if ((tid & 31) == 0) ws[tid >> 5] = t;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) tot += ws[w];
    *out = tot;
  }
}

}  // namespace gr
