// Per-atom regularisers of the fitting loops (sm_103a), in FP64.
//
// The reference's regularisers (GaussDictCode/regularisation.py:41-442) are
// closed forms of one atom's parameters; its Newton loop adds the gradient
// and Hessian of the regulariser to each atom's block
// (NewtonGaussian.py:59-66) and adds its value to the energy.  Here one thread
// per atom evaluates value, gradient (P) and Hessian (P x P) in the
// parameter order [I, x, r] and writes or adds them into the same arrays the
// derivative kernels fill, so a batched Newton step regularises every atom
// in one launch.
//
// With D the dimension, "diag r" the first D entries of an anisotropic r
// (the diagonal of the triangular factor) and s the isotropic r:
//   Joubert  -a log I + b/2 |x|^2 + c R - d log R - e,
//            R = prod(diag r) (aniso) or s^D (iso)          (:41-107)
//   Mass     w (I V - m)^k, V = 1/prod(diag r) or s^D       (:110-208)
//   Volume   w |R - v0|^k, R = prod(diag r) or s^-D         (:211-297)
//   Radius   w sum_i (r_i - r0)^-k over diag r (iso: D (s - r0)^-k) (:300-366)
//   Iso      w/2 |off-diagonal r|^2                           (:369-442)
// Values outside the domain the reference rejects (log or power of a
// non-positive number) are +inf, as there.  Hessians are the exact second
// derivatives of these values (the reference's Joubert has none, its Volume
// Hessian cannot run and its Mass Hessian misses mixed r-r terms).
#include <cmath>

#include "gr_kernels.cuh"
#include "gauss_radon.h"

namespace gr {

enum RegKind : int { kRegNull = 0, kRegJoubert = 1, kRegMass = 2, kRegVolume = 3,
                     kRegRadius = 4, kRegIso = 5 };

template <int D>
__global__ void __launch_bounds__(128)
    gr_reg_kernel(int kind, RegParams prm, int n, int iso, const float *Iv, const float *xv,
                  const float *rv, double *f, double *g, double *H, int accumulate) {
  constexpr int PR = D == 2 ? 3 : 6;
  constexpr int PMAX = 1 + D + PR;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int pr = iso ? 1 : PR;
  const int P = 1 + D + pr;
  const int r0 = 1 + D;  // first r parameter
  double gl[PMAX], hl[PMAX][PMAX];
  for (int a = 0; a < PMAX; ++a) {
    gl[a] = 0.0;
    for (int b = 0; b < PMAX; ++b) hl[a][b] = 0.0;
  }
  double val = 0.0;
  const double I = Iv[j];
  double x[D], r[PR];
  for (int c = 0; c < D; ++c) x[c] = xv[(size_t)j * D + c];
  for (int q = 0; q < pr; ++q) r[q] = rv[(size_t)j * pr + q];
  const double inf = HUGE_VAL;
  const int nd = iso ? 1 : D;  // r parameters that enter R

  if (kind == kRegJoubert) {
    const double a = prm.p[0], b = prm.p[1], c = prm.p[2], d = prm.p[3], e = prm.p[4];
    bool ok = I > 0.0;
    double R = 1.0;
    if (iso) {
      ok = ok && r[0] > 0.0;
      R = pow(r[0], (double)D);
    } else {
      for (int q = 0; q < D; ++q) {
        ok = ok && r[q] > 0.0;
        R *= r[q];
      }
    }
    double xx = 0.0;
    for (int c2 = 0; c2 < D; ++c2) xx += x[c2] * x[c2];
    val = ok ? (-a * log(I) + 0.5 * b * xx + c * R - d * log(R) - e) : inf;
    gl[0] = -a / I;
    hl[0][0] = a / (I * I);
    for (int c2 = 0; c2 < D; ++c2) {
      gl[1 + c2] = b * x[c2];
      hl[1 + c2][1 + c2] = b;
    }
    if (iso) {
      const double s = r[0];
      gl[r0] = D * c * pow(s, D - 1.0) - D * d / s;
      hl[r0][r0] = D * (D - 1.0) * c * pow(s, D - 2.0) + D * d / (s * s);
    } else {
      for (int q = 0; q < D; ++q) {
        gl[r0 + q] = (c * R - d) / r[q];
        for (int t = 0; t < D; ++t)
          hl[r0 + q][r0 + t] = (q == t) ? d / (r[q] * r[q]) : c * R / (r[q] * r[t]);
      }
    }
  } else if (kind == kRegMass) {
    const double m = prm.p[0], k = prm.p[1], w = prm.p[2];
    // V = I * Rv; dV and d2V over the parameters [I, r...]
    double Rv = 1.0;
    if (iso) Rv = pow(r[0], (double)D);
    else
      for (int q = 0; q < D; ++q) Rv /= r[q];
    const double V = I * Rv;
    double dV[PMAX], d2V[PMAX][PMAX];
    for (int a2 = 0; a2 < PMAX; ++a2) {
      dV[a2] = 0.0;
      for (int b2 = 0; b2 < PMAX; ++b2) d2V[a2][b2] = 0.0;
    }
    dV[0] = Rv;
    if (iso) {
      const double s = r[0];
      dV[r0] = D * I * pow(s, D - 1.0);
      d2V[0][r0] = d2V[r0][0] = D * pow(s, D - 1.0);
      d2V[r0][r0] = D * (D - 1.0) * I * pow(s, D - 2.0);
    } else {
      for (int q = 0; q < D; ++q) {
        dV[r0 + q] = -V / r[q];
        d2V[0][r0 + q] = d2V[r0 + q][0] = -Rv / r[q];
        for (int t = 0; t < D; ++t)
          d2V[r0 + q][r0 + t] = (q == t ? 2.0 : 1.0) * V / (r[q] * r[t]);
      }
    }
    const double u = V - m;
    val = (I < 0.0) ? inf : w * pow(fabs(V) - m, k);
    const double s1 = w * k * pow(u, k - 1.0);
    const double s2 = w * k * (k - 1.0) * pow(u, k - 2.0);
    for (int a2 = 0; a2 < P; ++a2) {
      gl[a2] = s1 * dV[a2];
      for (int b2 = 0; b2 < P; ++b2) hl[a2][b2] = s2 * dV[a2] * dV[b2] + s1 * d2V[a2][b2];
    }
  } else if (kind == kRegVolume) {
    const double v0 = prm.p[0], k = prm.p[1], w = prm.p[2];
    double R = 1.0, dR[PR], d2R[PR][PR];
    bool ok = true;
    for (int q = 0; q < PR; ++q) {
      dR[q] = 0.0;
      for (int t = 0; t < PR; ++t) d2R[q][t] = 0.0;
    }
    if (iso) {
      const double s = r[0];
      ok = s > 0.0;
      R = pow(s, -(double)D);
      dR[0] = -D * pow(s, -D - 1.0);
      d2R[0][0] = D * (D + 1.0) * pow(s, -D - 2.0);
    } else {
      for (int q = 0; q < D; ++q) {
        ok = ok && r[q] > 0.0;
        R *= r[q];
      }
      for (int q = 0; q < D; ++q) {
        dR[q] = R / r[q];
        for (int t = 0; t < D; ++t) d2R[q][t] = (q == t) ? 0.0 : R / (r[q] * r[t]);
      }
    }
    const double u = R - v0, au = fabs(u), sg = u > 0.0 ? 1.0 : (u < 0.0 ? -1.0 : 0.0);
    val = ok ? w * pow(au, k) : inf;
    const double s1 = w * k * sg * pow(au, k - 1.0);
    const double s2 = w * k * (k - 1.0) * pow(au, k - 2.0);
    for (int q = 0; q < nd; ++q) {
      gl[r0 + q] = s1 * dR[q];
      for (int t = 0; t < nd; ++t) hl[r0 + q][r0 + t] = s2 * dR[q] * dR[t] + s1 * d2R[q][t];
    }
  } else if (kind == kRegRadius) {
    const double rr0 = prm.p[0], w = prm.p[1], k = prm.p[2];
    const double mult = iso ? (double)D : 1.0;
    bool ok = true;
    for (int q = 0; q < nd; ++q) {
      const double t = r[q] - rr0;
      ok = ok && t > 0.0;
      val += mult * pow(t, -k);
      gl[r0 + q] = w * mult * (-k) * pow(t, -k - 1.0);
      hl[r0 + q][r0 + q] = w * mult * k * (k + 1.0) * pow(t, -k - 2.0);
    }
    val = ok ? w * val : inf;
  } else if (kind == kRegIso) {
    const double w = prm.p[0];
    if (!iso) {
      for (int q = D; q < PR; ++q) {
        val += 0.5 * w * r[q] * r[q];
        gl[r0 + q] = w * r[q];
        hl[r0 + q][r0 + q] = w;
      }
    }
  }

  if (f) f[j] = accumulate ? f[j] + val : val;
  for (int a2 = 0; a2 < P; ++a2) {
    double *gp = g + (size_t)j * P + a2;
    *gp = accumulate ? *gp + gl[a2] : gl[a2];
    if (H)
      for (int b2 = 0; b2 < P; ++b2) {
        double *hp = H + ((size_t)j * P + a2) * P + b2;
        *hp = accumulate ? *hp + hl[a2][b2] : hl[a2][b2];
      }
  }
}

int launch_regulariser(int kind, const RegParams &prm, int dim, int iso, int n,
                       const float *I, const float *x, const float *r, double *f, double *g,
                       double *H, int accumulate, cudaStream_t stream) {
  if (kind < kRegNull || kind > kRegIso || (dim != 2 && dim != 3) || n < 0) return kErrArg;
  if (n == 0) return kOk;
  if (!I || !x || !r || !g) return kErrArg;
  const int blocks = (n + 127) / 128;
  if (dim == 2)
    gr_reg_kernel<2><<<blocks, 128, 0, stream>>>(kind, prm, n, iso, I, x, r, f, g, H, accumulate);
  else
    gr_reg_kernel<3><<<blocks, 128, 0, stream>>>(kind, prm, n, iso, I, x, r, f, g, H, accumulate);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int preload_reg() { return preload_fn(gr_reg_kernel<2>) + preload_fn(gr_reg_kernel<3>); }

}  // namespace gr

extern "C" int gr_regulariser(int kind, const double *params, int n_params,
                              const gr_atoms *atoms, int dim, double *f, double *g, double *H,
                              int accumulate, void *stream) {
  if (!atoms || (n_params > 0 && !params) || n_params < 0 || n_params > 8) return gr::kErrArg;
  gr::RegParams prm;
  for (int i = 0; i < 8; ++i) prm.p[i] = i < n_params ? params[i] : 0.0;
  return gr::launch_regulariser(kind, prm, dim, atoms->r_iso, atoms->n_atoms, atoms->I, atoms->x,
                                atoms->r, f, g, H, accumulate,
                                static_cast<cudaStream_t>(stream));
}
