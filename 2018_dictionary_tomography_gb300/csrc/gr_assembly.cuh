// Chain-rule assembly of per-atom gradients and Hessians from psi-space
// sums, shared by the point-sampled (gr_derivs.cu) and pixel-integrated
// (gr_psf.cu) derivative kernels.  See gr_derivs.cu for the derivation.
#pragma once
#include "gr_kernels.cuh"

namespace gr {

template <int K>
__host__ __device__ constexpr int n_psi() { return 1 + K * (K + 1) / 2 + K; }
template <int K>
__host__ __device__ constexpr int n_par() { return 1 + (K + 1) + n_rparam<K>(); }  // I, x, r
template <int K, int DEG>
__host__ __device__ constexpr int n_mom() { return K == 1 ? DEG + 1 : (DEG + 1) * (DEG + 2) / 2; }
// monomial d0^i d1^j -> moment slot (ordered by total degree)
__host__ __device__ constexpr int mi(int i, int j) {
  return (i + j) * (i + j + 1) / 2 + j;
}

// Basis vector c of the frame: detector axes 0..K-1, then the ray direction.
template <int K>
__device__ __forceinline__ float basis(const Frame<K> &f, int c, int b) {
  return c < K ? f.w[c][b] : f.T[b];
}

// A_psi = sum w dl/dpsi from moments (psi order: ln n, G params, q*).
template <int K, int NM>
__device__ __forceinline__ void first_psi(const float *M, const float *G,
                                          float *A) {
  A[0] = M[0];
  if constexpr (K == 1) {
    A[1] = -30.f * M[2];
    A[2] = 60.f * G[0] * M[1];
  } else {
    A[1] = -30.f * M[mi(2, 0)];
    A[2] = -60.f * M[mi(1, 1)];
    A[3] = -30.f * M[mi(0, 2)];
    A[4] = 60.f * (G[0] * M[mi(1, 0)] + G[1] * M[mi(0, 1)]);
    A[5] = 60.f * (G[1] * M[mi(1, 0)] + G[2] * M[mi(0, 1)]);
  }
}

// Gradient of sum_psi A_psi psi with respect to (x, r), times scale:
// x part through q* = B^{-1} x, r part through Q = (rB)^T(rB) via the
// adjoint Abar of psi(Q): d/dr_(ab) = 2 (Kc^T Abar B^T)_ab.
template <int K>
__device__ __forceinline__ void psi_grad(const Pair<K> &p, const Frame<K> &f,
                                         const float *A, float *gx, float *gr) {
  constexpr int D = K + 1;
  constexpr int NG = K * (K + 1) / 2;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < K; ++i) s = fmaf(A[1 + NG + i], f.wt[i][c], s);
    gx[c] = s;
  }
  const float iq = 1.f / p.Q[K][K];
  float Ah[K][K];
  if constexpr (K == 1) {
    Ah[0][0] = A[1];
  } else {
    Ah[0][0] = A[1];
    Ah[0][1] = 0.5f * A[2];
    Ah[1][0] = 0.5f * A[2];
    Ah[1][1] = A[3];
  }
  float Ab[D][D];
  float hAh = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      Ab[i][j] = Ah[i][j];
      s = fmaf(Ah[i][j], p.Q[j][K], s);
    }
    Ab[i][K] = -s * iq;
    Ab[K][i] = -s * iq;
    hAh = fmaf(p.Q[i][K], s, hAh);
  }
  Ab[K][K] = hAh * iq * iq - 0.5f * A[0] * iq;
  // Y = Abar B^T, X = Kc^T Y
  float Y[D][D];
#pragma unroll
  for (int d = 0; d < D; ++d)
#pragma unroll
    for (int b = 0; b < D; ++b) {
      float s = 0.f;
#pragma unroll
      for (int c = 0; c < D; ++c) s = fmaf(Ab[d][c], basis<K>(f, c, b), s);
      Y[d][b] = s;
    }
#pragma unroll
  for (int q = 0; q < n_rparam<K>(); ++q) {
    const int a = rrow<K>(q), b = rcol<K>(q);
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d) s = fmaf(p.Kc[d][a], Y[d][b], s);
    gr[q] = 2.f * s;
  }
}

// psi-space Gram matrix of the cell weights:
// out[k][l] = sum w dl/dpsi_k dl/dpsi_l (+ sum w d2l/dpsi_k dpsi_l if WITH_C).
template <int K, bool WITH_C>
__device__ __forceinline__ void psi_gram(const float *M, const float *G,
                                         float (&B)[n_psi<K>()][n_psi<K>()]) {
  if constexpr (K == 1) {
    const float g = G[0];
    B[0][0] = M[0];
    B[0][1] = -30.f * M[2];
    B[0][2] = 60.f * g * M[1];
    B[1][1] = 900.f * M[4];
    B[1][2] = -1800.f * g * M[3];
    B[2][2] = 3600.f * g * g * M[2];
    if (WITH_C) {
      B[2][2] += -60.f * g * M[0];
      B[1][2] += 60.f * M[1];
    }
  } else {
    const float g0 = G[0], g1 = G[1], g2 = G[2];
    B[0][0] = M[mi(0, 0)];
    B[0][1] = -30.f * M[mi(2, 0)];
    B[0][2] = -60.f * M[mi(1, 1)];
    B[0][3] = -30.f * M[mi(0, 2)];
    B[0][4] = 60.f * (g0 * M[mi(1, 0)] + g1 * M[mi(0, 1)]);
    B[0][5] = 60.f * (g1 * M[mi(1, 0)] + g2 * M[mi(0, 1)]);
    B[1][1] = 900.f * M[mi(4, 0)];
    B[1][2] = 1800.f * M[mi(3, 1)];
    B[1][3] = 900.f * M[mi(2, 2)];
    B[1][4] = -1800.f * (g0 * M[mi(3, 0)] + g1 * M[mi(2, 1)]);
    B[1][5] = -1800.f * (g1 * M[mi(3, 0)] + g2 * M[mi(2, 1)]);
    B[2][2] = 3600.f * M[mi(2, 2)];
    B[2][3] = 1800.f * M[mi(1, 3)];
    B[2][4] = -3600.f * (g0 * M[mi(2, 1)] + g1 * M[mi(1, 2)]);
    B[2][5] = -3600.f * (g1 * M[mi(2, 1)] + g2 * M[mi(1, 2)]);
    B[3][3] = 900.f * M[mi(0, 4)];
    B[3][4] = -1800.f * (g0 * M[mi(1, 2)] + g1 * M[mi(0, 3)]);
    B[3][5] = -1800.f * (g1 * M[mi(1, 2)] + g2 * M[mi(0, 3)]);
    B[4][4] = 3600.f * (g0 * g0 * M[mi(2, 0)] + 2.f * g0 * g1 * M[mi(1, 1)] +
                        g1 * g1 * M[mi(0, 2)]);
    B[4][5] = 3600.f * (g0 * g1 * M[mi(2, 0)] + (g0 * g2 + g1 * g1) * M[mi(1, 1)] +
                        g1 * g2 * M[mi(0, 2)]);
    B[5][5] = 3600.f * (g1 * g1 * M[mi(2, 0)] + 2.f * g1 * g2 * M[mi(1, 1)] +
                        g2 * g2 * M[mi(0, 2)]);
    if (WITH_C) {
      B[4][4] += -60.f * g0 * M[0];
      B[4][5] += -60.f * g1 * M[0];
      B[5][5] += -60.f * g2 * M[0];
      B[1][4] += 60.f * M[mi(1, 0)];
      B[2][4] += 60.f * M[mi(0, 1)];
      B[2][5] += 60.f * M[mi(1, 0)];
      B[3][5] += 60.f * M[mi(0, 1)];
    }
  }
#pragma unroll
  for (int i = 0; i < n_psi<K>(); ++i)
#pragma unroll
    for (int j = 0; j < i; ++j) B[i][j] = B[j][i];
}

// Jacobian of (ln n, G params) with respect to r, and
// sum_psi A_psi d2 psi / dr dr (Hr, packed upper triangle).
template <int K>
__device__ __forceinline__ void psi_r_derivs(
    const Pair<K> &p, const Frame<K> &f, const float *A,
    float (&Jr)[1 + K * (K + 1) / 2][n_rparam<K>()],
    float (&Hr)[n_rparam<K>() * (n_rparam<K>() + 1) / 2]) {
  constexpr int D = K + 1;
  constexpr int PR = n_rparam<K>();
  constexpr int NG = K * (K + 1) / 2;
  constexpr int NE = NG + K + 1;  // distinct Q entries: G entries, (m, T), (T, T)
  const float w = p.Q[K][K], iq = 1.f / w;
  // entry e = (ec, ed): the NG detector pairs in G order, then (m, T), (T, T)
  int ec[NE], ed[NE];
  if constexpr (K == 1) {
    ec[0] = 0; ed[0] = 0;
    ec[1] = 0; ed[1] = 1;
    ec[2] = 1; ed[2] = 1;
  } else {
    ec[0] = 0; ed[0] = 0;
    ec[1] = 0; ed[1] = 1;
    ec[2] = 1; ed[2] = 1;
    ec[3] = 0; ed[3] = 2;
    ec[4] = 1; ed[4] = 2;
    ec[5] = 2; ed[5] = 2;
  }
  // DQ[e][q] = dQ_e / dr_q = B_c[b] K_d[a] + B_d[b] K_c[a], r_q = r_ab
  float DQ[NE][PR];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int q = 0; q < PR; ++q) {
      const int a = rrow<K>(q), b = rcol<K>(q);
      DQ[e][q] = basis<K>(f, ec[e], b) * p.Kc[ed[e]][a] + basis<K>(f, ed[e], b) * p.Kc[ec[e]][a];
    }
  float uT[K];
#pragma unroll
  for (int m = 0; m < K; ++m) uT[m] = p.Q[m][K];
  // first derivatives: psi_0 = ln n = -ln(Q_TT)/2, G_ij = Q_ij - Q_iT Q_jT / Q_TT
#pragma unroll
  for (int q = 0; q < PR; ++q) Jr[0][q] = -0.5f * DQ[NE - 1][q] * iq;
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    const int i = ec[k], j = ed[k];
#pragma unroll
    for (int q = 0; q < PR; ++q)
      Jr[1 + k][q] = DQ[k][q] - (DQ[NG + i][q] * uT[j] + uT[i] * DQ[NG + j][q]) * iq +
                     uT[i] * uT[j] * DQ[NE - 1][q] * iq * iq;
  }
  // Second derivatives of Psi = sum_k A_k psi_k through the entries of Q:
  //   d2Psi/dr dr = DQ^T (d2Psi/dQ dQ) DQ + [same row of r] (B^T Abar B)
  // with Abar = dPsi/dQ; d2Psi/dQ dQ is non-zero only among the (m, T) and
  // (T, T) entries.
  float Abar[NE], A2[K + 1][K + 1];
  float sg = 0.f;  // sum_k A_k Q_iT Q_jT
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    Abar[k] = A[1 + k];
    sg = fmaf(A[1 + k], uT[ec[k]] * uT[ed[k]], sg);
  }
#pragma unroll
  for (int m = 0; m < K; ++m) {
    float t = 0.f;  // sum_k A_k dG_k/dQ_mT * (-Q_TT)
#pragma unroll
    for (int k = 0; k < NG; ++k)
      t += A[1 + k] * ((ec[k] == m ? uT[ed[k]] : 0.f) + (ed[k] == m ? uT[ec[k]] : 0.f));
    Abar[NG + m] = -t * iq;
    A2[m][K] = A2[K][m] = t * iq * iq;
#pragma unroll
    for (int n = 0; n < K; ++n) {
      float t2 = 0.f;
#pragma unroll
      for (int k = 0; k < NG; ++k)
        t2 += A[1 + k] * (((ec[k] == m && ed[k] == n) ? 1.f : 0.f) +
                          ((ed[k] == m && ec[k] == n) ? 1.f : 0.f));
      A2[m][n] = -t2 * iq;
    }
  }
  Abar[NE - 1] = sg * iq * iq - 0.5f * A[0] * iq;
  A2[K][K] = -2.f * sg * iq * iq * iq + 0.5f * A[0] * iq * iq;
  // M = sum_e Abar_e (B_c B_d^T + B_d B_c^T)
  float M[D][D];
#pragma unroll
  for (int b = 0; b < D; ++b)
#pragma unroll
    for (int b2 = 0; b2 < D; ++b2) {
      float t = 0.f;
#pragma unroll
      for (int e = 0; e < NE; ++e)
        t = fmaf(Abar[e], basis<K>(f, ec[e], b) * basis<K>(f, ed[e], b2) +
                              basis<K>(f, ed[e], b) * basis<K>(f, ec[e], b2), t);
      M[b][b2] = t;
    }
  // Y = (d2Psi/dQ_T dQ_T) DQ_T
  float Y[K + 1][PR];
#pragma unroll
  for (int e = 0; e <= K; ++e)
#pragma unroll
    for (int s2 = 0; s2 < PR; ++s2) {
      float t = 0.f;
#pragma unroll
      for (int e2 = 0; e2 <= K; ++e2) t = fmaf(A2[e][e2], DQ[NG + e2][s2], t);
      Y[e][s2] = t;
    }
  int o = 0;
#pragma unroll
  for (int q = 0; q < PR; ++q)
#pragma unroll
    for (int s2 = q; s2 < PR; ++s2, ++o) {
      float h = (rrow<K>(q) == rrow<K>(s2)) ? M[rcol<K>(q)][rcol<K>(s2)] : 0.f;
#pragma unroll
      for (int e = 0; e <= K; ++e) h = fmaf(DQ[NG + e][q], Y[e][s2], h);
      Hr[o] = h;
    }
}

// Adds one (atom, angle) pair's contribution to the per-atom gradient and
// (ORDER 2) packed Hessian over (I, x, r), from its psi-space sums:
//   Aa[k]    = sum alpha * dl/dpsi_k           (weights alpha * E)
//   Ba[k][l] = sum alpha * (dl_k dl_l + d2l_kl) (ORDER 2)
//   Bb[k][l] = sum beta * dR dR^T in psi space  (Gauss-Newton part, ORDER 2;
//              Bb[0][k] is its I-row)
// with the chain rule psi -> (I, x, r) of gr_common.cuh.
template <int K, int ORDER>
__device__ __forceinline__ void accumulate_pair(
    const Pair<K> &p, const Frame<K> &fr, float I, const float *Aa,
    const float (&Ba)[n_psi<K>()][n_psi<K>()], const float (&Bb)[n_psi<K>()][n_psi<K>()],
    CAcc *gacc, float *hacc) {
  constexpr int D = K + 1;
  constexpr int PR = n_rparam<K>();
  constexpr int NPSI = n_psi<K>();
  constexpr int NG = K * (K + 1) / 2;
  // gradient: g_I = sum alpha E, g_xi = I sum_psi A_psi dpsi/dxi
  float gx[D], grr[PR];
  psi_grad<K>(p, fr, Aa, gx, grr);
  gacc[0].add(Aa[0]);
#pragma unroll
  for (int c = 0; c < D; ++c) gacc[1 + c].add(I * gx[c]);
#pragma unroll
  for (int q = 0; q < PR; ++q) gacc[1 + D + q].add(I * grr[q]);
  if constexpr (ORDER > 1) {
    float Ab[NPSI];
#pragma unroll
    for (int k = 0; k < NPSI; ++k) Ab[k] = Bb[0][k];
    float X[NPSI][NPSI];
#pragma unroll
    for (int k = 0; k < NPSI; ++k)
#pragma unroll
      for (int l = 0; l < NPSI; ++l) X[k][l] = I * Ba[k][l] + I * I * Bb[k][l];
    float Jr[1 + NG][PR];
    float Hr[PR * (PR + 1) / 2];
    psi_r_derivs<K>(p, fr, Aa, Jr, Hr);
    // mixed first-order terms for the I row
    float Am[NPSI];
#pragma unroll
    for (int k = 0; k < NPSI; ++k) Am[k] = Aa[k] + I * Ab[k];
    float hx[D], hr[PR];
    psi_grad<K>(p, fr, Am, hx, hr);
    // packed upper triangle over (I, x, r)
    int o = 0;
    hacc[o++] += Bb[0][0];  // (I, I)
#pragma unroll
    for (int c = 0; c < D; ++c) hacc[o++] += hx[c];
#pragma unroll
    for (int q = 0; q < PR; ++q) hacc[o++] += hr[q];
    // x rows
#pragma unroll
    for (int c = 0; c < D; ++c) {
#pragma unroll
      for (int c2 = c; c2 < D; ++c2) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
          for (int i2 = 0; i2 < K; ++i2)
            s = fmaf(fr.wt[i][c] * X[1 + NG + i][1 + NG + i2], fr.wt[i2][c2], s);
        hacc[o++] += s;
      }
#pragma unroll
      for (int q = 0; q < PR; ++q) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < K; ++i) {
          float t = 0.f;
#pragma unroll
          for (int k = 0; k < 1 + NG; ++k) t = fmaf(X[1 + NG + i][k], Jr[k][q], t);
          s = fmaf(fr.wt[i][c], t, s);
        }
        hacc[o++] += s;
      }
    }
    // r rows
    int hro = 0;
#pragma unroll
    for (int q = 0; q < PR; ++q)
#pragma unroll
      for (int s2 = q; s2 < PR; ++s2, ++hro) {
        float s = I * Hr[hro];
#pragma unroll
        for (int k = 0; k < 1 + NG; ++k) {
          float t = 0.f;
#pragma unroll
          for (int l = 0; l < 1 + NG; ++l) t = fmaf(X[k][l], Jr[l][s2], t);
          s = fmaf(Jr[k][q], t, s);
        }
        hacc[o++] += s;
      }
  }
}

}  // namespace gr
