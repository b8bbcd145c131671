// Per-atom derivatives of data fits (sm_103a).
//
// Replaces the reference's one-atom-per-launch kernels
// __L2derivs_RadProj_aniso (GaussDictCode/bin/NewtonBases2D.py:331-401),
// __derivs_RadProj_aniso (NewtonBases2D.py:446-515) and their 3D twins
// (GaussDictCode/bin/NewtonBases.py:794-870, :995-1069), which evaluate a
// 6x6 / 10x10 per-cell Hessian of one atom at every detector cell.
//
// For one (atom, angle) pair the projection is R(q) = I E(q),
// E = n exp(-30 (q - q*)^T G (q - q*)) (see gr_common.cuh), so
//   ln E = ln n - 30 d^T G d,   d = q - q*,
// is linear in psi = (ln n, G, q*) up to the quadratic dependence on q*.
// Every derivative sum over cells of a weight field w times a polynomial in d
// is therefore a combination of a few cell moments  M_ij = sum w d0^i d1^j
// (degree <= 2 for gradients, <= 4 for Hessians), and the chain rule from psi
// to (I, x, r) is done once per pair:
//   psi -> Q = (r B)^T (r B) -> r   and   q* = (B^{-1} x)[0:K].
// Per cell the kernel evaluates one exp2 and a handful of FMAs; moments are
// accumulated per detector row and folded with powers of d0 at row end.
//
// Work layout: lane = atom, a warp holds 32 atoms (or fewer atoms with the
// angles of each atom split over several lanes), and loops over a chunk of
// angles.  Gradients are accumulated per lane with compensated FP32 sums,
// Hessians in FP32; lanes sharing an atom are combined by a fixed-order
// butterfly; chunk partials are summed in FP64 in chunk order by
// gr_deriv_finalize_kernel, which also applies the isotropic chain rule.
// No float atomics anywhere: results are bitwise reproducible.
#include "gr_assembly.cuh"

namespace gr {

inline int next_pow2(int v) {
  int p = 1;
  while (p < v && p < 32) p <<= 1;
  return p;
}

constexpr int kRowChunk = 8;
// cells per chunk of a 3D box row, and resident blocks per SM asked of the
// gradient (order 1) kernels; compile-time, for sweeps
// (4 and 8 measured best on 8192 atoms x 5000 orientations: 4.59 ms against
// 5.73 ms for 8-cell chunks at 5 blocks; 64 registers, with a few spills,
// give the gradient kernels 32 resident warps per SM instead of 20)
#ifndef GR_ROW_CHUNK_3D
#define GR_ROW_CHUNK_3D 4
#endif
#ifndef GR_GRAD_MIN_BLOCKS
#define GR_GRAD_MIN_BLOCKS 8
#endif
// resident blocks per SM asked of the 2D Hessian kernel with one angle per lane
#ifndef GR_HESS2D_MIN_BLOCKS
#define GR_HESS2D_MIN_BLOCKS 3
#endif
constexpr int kRowChunk3 = GR_ROW_CHUNK_3D;

// Work split of the derivative kernels (Tuning, gr_set_tuning / gr_plan_set):
// about deriv_target_warps warps in total, each angle chunk holding at least
// deriv_min_angles angles per lane group.
// deriv_atoms_per_warp (power of two up to 32; 0 = automatic): with fewer
// atoms per warp the lanes of a warp take different angles of one atom, whose
// support boxes are of similar size, so fewer lanes idle.  Automatic: one
// atom per warp for Hessians and for long angle series, else four (so each
// lane still has a few angles to amortise the warp's closing reduction).
// deriv_split_lanes: problems with few (atom, angle) pairs split each pair's
// cells over rs lanes (rows of a 3D box, chunks of kRowChunk cells of a 2D
// one), rs the largest power of two up to 8 with pairs * rs <=
// deriv_split_lanes; the lanes' moment sums are combined before one of them
// does the chain-rule assembly.  A pair's cell walk is otherwise one lane's
// serial loop, which sets the kernel time when there are too few pairs to
// fill the GPU and their boxes are large.  0: never split.
// deriv_one_mb: take as many angle chunks as give every lane at most one
// angle (the ONE kernel variant: fewer registers, no spills) whenever the
// chunk partials then fit in this many MB; 0: keep the target-warps split.
// On 8192 atoms x 20000 orientations the one-angle split (625 chunks, 225 MB
// of partials) runs the gradient kernel in 23.6 ms against 25.7 ms for 16
// chunks.
DerivCfg deriv_cfg(int K, int n_atoms, int n_angles, int order, const Tuning &t, bool split) {
  DerivCfg c;
  c.ag = next_pow2(n_atoms < 1 ? 1 : n_atoms);
  const int ag_cap = t.deriv_atoms_per_warp > 0 ? t.deriv_atoms_per_warp
                     : (order > 1 || n_angles >= 1024) ? 1 : 4;
  if (c.ag > ag_cap) c.ag = ag_cap;
  c.sg = 32 / c.ag;
  const long long pairs = (long long)(n_atoms < 1 ? 1 : n_atoms) * (n_angles < 1 ? 1 : n_angles);
  c.rs = 1;
  while (split && t.deriv_split_lanes > 0 && c.rs < 8 && c.rs < c.sg &&
         pairs * c.rs * 2 <= (long long)t.deriv_split_lanes)
    c.rs <<= 1;
  const int warps_atoms = (n_atoms + c.ag - 1) / c.ag;
  int nch = (t.deriv_target_warps + warps_atoms - 1) / warps_atoms;
  const int per = (c.sg / c.rs) * (t.deriv_min_angles < 1 ? 1 : t.deriv_min_angles);
  const int max_ch = (n_angles + per - 1) / per;
  if (nch > max_ch) nch = max_ch;
  const int P0 = 1 + (K + 1) + (K == 1 ? 3 : 6);
  const size_t qn0 = 1 + P0 + (order > 1 ? P0 * (P0 + 1) / 2 : 0);
  if (t.deriv_one_mb > 0 && t.deriv_min_angles == 1 && nch < max_ch &&
      (size_t)max_ch * qn0 * (size_t)(n_atoms < 1 ? 1 : n_atoms) * sizeof(float) <=
          ((size_t)t.deriv_one_mb << 20))
    nch = max_ch;
  if (nch < 1) nch = 1;
  c.ch = (n_angles + nch - 1) / nch;
  if (c.ch < 1) c.ch = 1;
  c.nchunks = (n_angles + c.ch - 1) / c.ch;
  const int P = 1 + (K + 1) + (K == 1 ? 3 : 6);
  c.qn = 1 + P + (order > 1 ? P * (P + 1) / 2 : 0);
  return c;
}

// Cell moments of one pair.
template <int K, int DEG, bool GN>
struct PairMoments {
  float Ma[n_mom<K, DEG>()];
  float Mb[GN ? n_mom<K, DEG>() : 1];
  float X0, Y0;  // sum E*C and sum E^2 (per-atom L2 value)
};

// CH: cells per chunk of the row walk (loaded together before any is used)
template <int K, int DEG, bool GN, int CH>
__device__ __forceinline__ void pair_moments(const Pair<K> &p, const Geom &g,
                                             const DerivIn &in, int a, float I,
                                             PairMoments<K, DEG, GN> &mo, int phase = 0,
                                             int rs = 1) {
  constexpr int NM = n_mom<K, DEG>();
#pragma unroll
  for (int i = 0; i < NM; ++i) {
    mo.Ma[i] = 0.f;
    if (GN) mo.Mb[i] = 0.f;
  }
  mo.X0 = 0.f;
  mo.Y0 = 0.f;
  if (p.lo[0] > p.hi[0]) return;
  if constexpr (K == 2)
    if (p.lo[1] > p.hi[1]) return;
  const float l2n = lg2_approx(p.n);
  const int D0 = g.ax[0].n;
  const int D1 = K == 2 ? g.ax[1].n : 1;
  const float *__restrict__ field = in.alpha;
  const float *__restrict__ bfield = in.beta;
  const size_t abase = (size_t)a * D0 * D1;
  // per row, m <= 1 holds for d1 within hw(d0) = sqrt(G2 - d0^2 det)/G2 of
  // -G1 d0/G2: the row loop visits that range (widened like the support box)
  // instead of the whole box; the m <= 1 test still decides every cell
  float det = 0.f, iG2 = 0.f;
  if constexpr (K == 2) {
    det = p.G[0] * p.G[2] - p.G[1] * p.G[1];
    iG2 = 1.f / p.G[2];
  }
  if constexpr (K == 1) {
    // the detector row is walked in chunks of kRowChunk cells whose field
    // values and coordinates are loaded together first (one cell per load
    // round trip would leave the lane waiting on every cell)
    const int c_hi = p.hi[0];
    for (int kb = p.lo[0] + phase * CH; kb <= c_hi; kb += rs * CH) {
      float cv[CH], pv[CH], bv[GN ? CH : 1];
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        const int k0 = min(kb + i, c_hi);
        cv[i] = __ldg(field + abase + k0);
        pv[i] = __ldg(g.ax[0].coords + k0);
        if (GN) bv[i] = bfield ? __ldg(bfield + abase + k0) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        if (kb + i > c_hi) break;
        const float d0 = (pv[i] - p.qh[0]) - p.ql[0];
        const float m = p.G[0] * d0 * d0;
        if (m <= 1.f) {
          const float E = ex2_approx(fmaf(m, kNegThirtyLog2e, l2n));
          const float c = cv[i];
          const float al = (in.mode == kModeL2Atom) ? fmaf(I, E, -c) : c;
          // powers of d0, shared by both moment sets: one FMA per moment
          float pw[NM];
          pw[0] = 1.f;
#pragma unroll
          for (int q = 1; q < NM; ++q) pw[q] = pw[q - 1] * d0;
          const float w = al * E;
          mo.Ma[0] += w;
#pragma unroll
          for (int q = 1; q < NM; ++q) mo.Ma[q] = fmaf(w, pw[q], mo.Ma[q]);
          if (GN) {
            // a constant beta scales the moments once per pair instead
            const float wb = bfield ? bv[i] * (E * E) : E * E;
            mo.Mb[0] += wb;
#pragma unroll
            for (int q = 1; q < NM; ++q) mo.Mb[q] = fmaf(wb, pw[q], mo.Mb[q]);
          }
          if (in.mode == kModeL2Atom) {
            mo.X0 = fmaf(E, c, mo.X0);
            mo.Y0 = fmaf(E, E, mo.Y0);
          }
        }
      }
    }
  } else {
    for (int k0 = p.lo[0] + phase; k0 <= p.hi[0]; k0 += rs) {
      const float d0 = (__ldg(g.ax[0].coords + k0) - p.qh[0]) - p.ql[0];
      {
        const float t0 = p.G[0] * d0 * d0;
        const float u = 2.f * p.G[1] * d0;
        float Sa[DEG + 1], Sb[GN ? DEG + 1 : 1];
#pragma unroll
        for (int q = 0; q <= DEG; ++q) {
          Sa[q] = 0.f;
          if (GN) Sb[q] = 0.f;
        }
        const size_t rbase = abase + (size_t)k0 * D1;
        const float rem = fmaf(-d0 * d0, det, p.G[2]);
        const float rc = (p.qh[1] - p.G[1] * d0 * iG2 - g.ax[1].first) * g.ax[1].inv_step;
        const float rh = sqrtf(fmaxf(rem, 0.f)) * iG2 * g.ax[1].inv_step * 1.0001f + 1e-3f;
        const float rlo = ceilf(rc - rh), rhi = floorf(rc + rh);
        const int c_lo = (int)fminf(fmaxf(rlo, (float)p.lo[1]), (float)p.hi[1] + 1.f);
        const int c_hi = (int)fmaxf(fminf(rhi, (float)p.hi[1]), (float)p.lo[1] - 1.f);
        // the row is walked in chunks of CH cells whose field values and
        // coordinates are loaded together first, so the loads overlap
        // instead of each cell waiting for its own
        for (int kb = c_lo; kb <= c_hi; kb += CH) {
          float cv[CH], pv[CH], bv[GN ? CH : 1];
#pragma unroll
          for (int i = 0; i < CH; ++i) {
            const int k1 = min(kb + i, c_hi);
            cv[i] = __ldg(field + rbase + k1);
            pv[i] = __ldg(g.ax[1].coords + k1);
            if (GN) bv[i] = bfield ? __ldg(bfield + rbase + k1) : 0.f;
          }
#pragma unroll
          for (int i = 0; i < CH; ++i) {
            if (kb + i > c_hi) break;
            const float d1 = (pv[i] - p.qh[1]) - p.ql[1];
            const float m = fmaf(d1, fmaf(p.G[2], d1, u), t0);
            if (m <= 1.f) {
              const float E = ex2_approx(fmaf(m, kNegThirtyLog2e, l2n));
              const float c = cv[i];
              const float al = (in.mode == kModeL2Atom) ? fmaf(I, E, -c) : c;
              float pw[DEG + 1];
              pw[0] = 1.f;
#pragma unroll
              for (int q = 1; q <= DEG; ++q) pw[q] = pw[q - 1] * d1;
              const float w = al * E;
              Sa[0] += w;
#pragma unroll
              for (int q = 1; q <= DEG; ++q) Sa[q] = fmaf(w, pw[q], Sa[q]);
              if (GN) {
                const float wb = bfield ? bv[i] * (E * E) : E * E;
                Sb[0] += wb;
#pragma unroll
                for (int q = 1; q <= DEG; ++q) Sb[q] = fmaf(wb, pw[q], Sb[q]);
              }
              if (in.mode == kModeL2Atom) {
                mo.X0 = fmaf(E, c, mo.X0);
                mo.Y0 = fmaf(E, E, mo.Y0);
              }
            }
          }
        }
        float pw = 1.f;
#pragma unroll
        for (int i = 0; i <= DEG; ++i) {
#pragma unroll
          for (int j = 0; j <= DEG - i; ++j) {
            mo.Ma[mi(i, j)] = fmaf(pw, Sa[j], mo.Ma[mi(i, j)]);
            if (GN) mo.Mb[mi(i, j)] = fmaf(pw, Sb[j], mo.Mb[mi(i, j)]);
          }
          pw *= d0;
        }
      }
    }
  }
  if (GN && !bfield) {
#pragma unroll
    for (int q = 0; q < NM; ++q) mo.Mb[q] *= in.beta_const;
  }
}

// ONE: the work split gives every lane at most one angle of its atom (every
// Hessian split of up to ~32 angles per chunk, which covers the tilt series
// and the served fits): the angle loop runs at most once, so the per-lane
// accumulators need not live across the whole pair computation, which cuts
// the Hessian kernel from 255 to 168 registers (3 resident blocks per SM
// instead of 2).
// WIDE (3D Hessians): rows walked in chunks of 8 cells instead of 4, which
// keeps more field loads in flight when supports are many cells wide and
// costs idle lanes on narrow ones (Tuning key 8; measured: 2936 atoms x 148
// angles of 493^2 cells 460 -> 408 us, config 2's atoms 192 -> 200 us; 16
// instead of 8 cells slowed every 2D Hessian measured, by up to 25 %)
// The body of one block whose first warp is warp0 of the launch's warps
// (warp w takes the w-th (atom group, angle chunk); a multi-problem launch
// maps its blocks to (problem, first warp)).  What a warp computes depends on
// its warp index only, so the block size changes no result.
template <int K, int ORDER, bool ONE, bool WIDE = false>
__device__ __forceinline__ void deriv_body(const Atoms &at, const Geom &g, const DerivIn &in,
                                           const DerivCfg &cfg, float *part, int warp0) {
  constexpr int D = K + 1;
  constexpr int PR = n_rparam<K>();
  constexpr int P = n_par<K>();
  constexpr int NPSI = n_psi<K>();
  constexpr int NG = K * (K + 1) / 2;
  constexpr int DEG = ORDER == 1 ? 2 : 4;
  constexpr int NH = P * (P + 1) / 2;
  constexpr bool GN = ORDER > 1;
  const int gw = warp0 + ((int)threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int warps_atoms = (at.n + cfg.ag - 1) / cfg.ag;
  if (gw >= warps_atoms * cfg.nchunks) return;
  const int chunk = gw / warps_atoms, wa = gw - chunk * warps_atoms;
  const int j = wa * cfg.ag + (lane % cfg.ag);   // slot
  const int sub = lane / cfg.ag;
  const bool valid = j < at.n;
  const int jj = valid ? (at.order ? at.order[j] : j) : 0;  // atom of the slot
  const float I = at.I[jj];
  const int a_lo = chunk * cfg.ch;
  const int a_hi = min(g.n_angles, a_lo + cfg.ch);

  float f = 0.f;
  CAcc gacc[P];
  float hacc[ORDER > 1 ? NH : 1];
#pragma unroll
  for (int i = 0; i < P; ++i) gacc[i].zero();
#pragma unroll
  for (int i = 0; i < (ORDER > 1 ? NH : 1); ++i) hacc[i] = 0.f;

  // lanes sharing a pair (cfg.rs of them, sub = s rs + phase) walk its rows
  // phase, phase + rs, ... and combine their moment sums
  const int phase = sub & (cfg.rs - 1);
  unsigned gmask = 0u;
  for (int o = 0; o < cfg.rs; ++o) gmask |= 1u << (lane + (o - phase) * cfg.ag);
  for (int a = a_lo + sub / cfg.rs; a < a_hi && valid; a += cfg.sg / cfg.rs) {
    Frame<K> fr;
    load_frame<K>(g.frames, a, fr);
    Pair<K> p;
    pair_setup<K>(at, jj, fr, g, p);
    PairMoments<K, DEG, GN> mo;
    static_assert(!WIDE || K == 2, "wide rows: 3D Hessians only");
    constexpr int CH = K == 1 ? kRowChunk : (WIDE ? 2 * kRowChunk3 : kRowChunk3);
    pair_moments<K, DEG, GN, CH>(p, g, in, a, I, mo, phase, cfg.rs);
    for (int o = 1; o < cfg.rs; o <<= 1) {
#pragma unroll
      for (int q = 0; q < n_mom<K, DEG>(); ++q) {
        mo.Ma[q] += __shfl_xor_sync(gmask, mo.Ma[q], o * cfg.ag);
        if (GN) mo.Mb[q] += __shfl_xor_sync(gmask, mo.Mb[q], o * cfg.ag);
      }
      mo.X0 += __shfl_xor_sync(gmask, mo.X0, o * cfg.ag);
      mo.Y0 += __shfl_xor_sync(gmask, mo.Y0, o * cfg.ag);
    }
    if (phase == 0) {
      float Aa[NPSI];
      first_psi<K, n_mom<K, DEG>()>(mo.Ma, p.G, Aa);
      // value
      if (in.mode == kModeInner) f += I * mo.Ma[0];
      else if (in.mode == kModeL2Atom) f += I * (0.5f * I * mo.Y0 - mo.X0);
      if constexpr (ORDER > 1) {
        float Ba[NPSI][NPSI], Bb[NPSI][NPSI];
        psi_gram<K, true>(mo.Ma, p.G, Ba);
        psi_gram<K, false>(mo.Mb, p.G, Bb);
        accumulate_pair<K, ORDER>(p, fr, I, Aa, Ba, Bb, gacc, hacc);
      } else {
        float Z[NPSI][NPSI];
        accumulate_pair<K, ORDER>(p, fr, I, Aa, Z, Z, gacc, hacc);
      }
    }
    if constexpr (ONE) break;
  }

  // combine lanes sharing an atom, then write
  float vals_f = f;
  float gv[P];
#pragma unroll
  for (int i = 0; i < P; ++i) gv[i] = gacc[i].get();
  if (ORDER > 1 && cfg.ag == 1) {
    // one atom per warp: a reduce-scatter leaves the warp sum of value
    // 32 c + lane of the atom's qn values in lane `lane` (chunk c), so every
    // lane stores one value; a full butterfly of every value on every lane
    // would cost qn * 5 shuffles per lane instead of 31 per 32 values
    constexpr int QN = 1 + P + (ORDER > 1 ? NH : 0);
    constexpr int NC = (QN + 31) / 32;
    float *dst = part + (size_t)chunk * cfg.qn * at.n + j;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      float v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int q = 32 * c + k;
        v[k] = q == 0 ? vals_f : (q <= P ? gv[q - 1] : (q < QN ? hacc[q - 1 - P] : 0.f));
      }
      warp_reduce_scatter32(v, lane);
      const int q = 32 * c + lane;
      if (valid && q < QN) dst[(size_t)q * at.n] = v[0];
    }
    return;
  }
  for (int off = cfg.ag; off < 32; off <<= 1) {
    vals_f += __shfl_xor_sync(0xffffffffu, vals_f, off);
#pragma unroll
    for (int i = 0; i < P; ++i) gv[i] += __shfl_xor_sync(0xffffffffu, gv[i], off);
    if constexpr (ORDER > 1) {
#pragma unroll
      for (int i = 0; i < NH; ++i) hacc[i] += __shfl_xor_sync(0xffffffffu, hacc[i], off);
    }
  }
  if (!valid || sub != 0) return;
  const size_t N = at.n;
  float *dst = part + (size_t)chunk * cfg.qn * N + j;
  dst[0] = vals_f;
#pragma unroll
  for (int i = 0; i < P; ++i) dst[(1 + i) * N] = gv[i];
  if constexpr (ORDER > 1) {
#pragma unroll
    for (int i = 0; i < NH; ++i) dst[(1 + P + i) * N] = hacc[i];
  }
}

// BW warps per block.  With one-warp blocks a warp that finishes frees its
// slot at once; with four, a block holds its slot until its slowest warp
// (the one with the widest supports) is done, which lowers the resident
// warps of the register-limited Hessian kernels (Tuning key 9).
template <int K, int ORDER, bool ONE, bool WIDE = false, int BW = 4>
__global__ void __launch_bounds__(BW * 32,
                                  (ORDER == 1 ? GR_GRAD_MIN_BLOCKS
                                              : (ONE ? (K == 1 ? GR_HESS2D_MIN_BLOCKS : 3) : 1)) *
                                      4 / BW)
    gr_deriv_kernel(Atoms at, Geom g, DerivIn in, DerivCfg cfg, float *part) {
  deriv_body<K, ORDER, ONE, WIDE>(at, g, in, cfg, part, (int)blockIdx.x * BW);
}

// Pixel-integrated operator: per cell, the quadrature points' moments give
// the cell's value R = I s sum E and its psi-space derivative sums
// A_cell = s first_psi(M), BC_cell = s psi_gram(M) (the quadrature points
// are fixed, as in the reference's __drf2/__drf3, which also give the
// "total mass" cells zero derivatives).  The pair's sums
//   Sa = sum alpha A_cell, Ta = sum alpha BC_cell, Ub = sum beta A_cell A_cell^T
// feed the same chain-rule assembly as the point-sampled kernel.
template <int K, int ORDER>
__global__ void __launch_bounds__(128)
    gr_psf_deriv_kernel(Atoms at, Geom g, DerivIn in, DerivCfg cfg, float *part, float s) {
  constexpr int D = K + 1;
  constexpr int P = n_par<K>();
  constexpr int NPSI = n_psi<K>();
  constexpr int DEG = ORDER == 1 ? 2 : 4;
  constexpr int NM = n_mom<K, DEG>();
  constexpr int NH = P * (P + 1) / 2;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int warps_atoms = (at.n + cfg.ag - 1) / cfg.ag;
  if (gw >= warps_atoms * cfg.nchunks) return;
  const int chunk = gw / warps_atoms, wa = gw - chunk * warps_atoms;
  const int j = wa * cfg.ag + (lane % cfg.ag);   // slot
  const int sub = lane / cfg.ag;
  const bool valid = j < at.n;
  const int jj = valid ? (at.order ? at.order[j] : j) : 0;  // atom of the slot
  const float I = at.I[jj];
  const int a_lo = chunk * cfg.ch;
  const int a_hi = min(g.n_angles, a_lo + cfg.ch);
  const int D0 = g.ax[0].n, D1 = K == 2 ? g.ax[1].n : 1;

  float f = 0.f;
  CAcc gacc[P];
  float hacc[ORDER > 1 ? NH : 1];
#pragma unroll
  for (int i = 0; i < P; ++i) gacc[i].zero();
#pragma unroll
  for (int i = 0; i < (ORDER > 1 ? NH : 1); ++i) hacc[i] = 0.f;

  for (int a = a_lo + sub; a < a_hi && valid; a += cfg.sg) {
    Frame<K> fr;
    load_frame<K>(g.frames, a, fr);
    Pair<K> p;
    const bool ok = pair_setup<K>(at, jj, fr, g, p);
    PsfPair<K> q;
    psf_setup<K>(at, jj, g, p, ok, s, q);
    const float l2n = lg2_approx(p.n);
    float Sa[NPSI], Ta[NPSI][NPSI], Ub[NPSI][NPSI];
#pragma unroll
    for (int k = 0; k < NPSI; ++k) {
      Sa[k] = 0.f;
#pragma unroll
      for (int l = 0; l < NPSI; ++l) {
        Ta[k][l] = 0.f;
        Ub[k][l] = 0.f;
      }
    }
    const int lo1 = K == 2 ? q.lo[K - 1] : 0, hi1 = K == 2 ? q.hi[K - 1] : 0;
    for (int k0 = q.lo[0]; k0 <= q.hi[0]; ++k0) {
      for (int k1 = lo1; k1 <= hi1; ++k1) {
        float dc[K], base[K], step[K];
        dc[0] = (__ldg(g.ax[0].coords + k0) - p.qh[0]) - p.ql[0];
        if constexpr (K == 2) dc[1] = (__ldg(g.ax[1].coords + k1) - p.qh[1]) - p.ql[1];
        const int kind = psf_cell_kind<K>(q, dc, s, base, step);
        if (kind == 0) continue;
        const size_t gi = ((size_t)a * D0 + k0) * D1 + k1;
        const float c = __ldg(in.alpha + gi);
        if (kind == 1) {
          const float R = q.total;
          if (in.mode == kModeInner) f = fmaf(c, R, f);
          else if (in.mode == kModeL2Atom) f += R * (0.5f * R - c);
          continue;
        }
        float M[NM];
#pragma unroll
        for (int i = 0; i < NM; ++i) M[i] = 0.f;
        float scale;
        if constexpr (K == 1) {
#pragma unroll
          for (int t = 1; t <= 11; ++t) {
            const float d = fmaf((float)t, step[0], base[0]);
            float w = ex2_approx(fmaf(p.G[0] * d * d, kNegThirtyLog2e, l2n));
#pragma unroll
            for (int e = 0; e < NM; ++e) {
              M[e] += w;
              w *= d;
            }
          }
          scale = 10.f * step[0] / 11.f;
        } else {
          for (int t = 1; t <= 11; ++t) {
            const float d0 = fmaf((float)t, step[0], base[0]);
            const float t0 = p.G[0] * d0 * d0, u = 2.f * p.G[1] * d0;
            float S[DEG + 1];
#pragma unroll
            for (int e = 0; e <= DEG; ++e) S[e] = 0.f;
            for (int v = 1; v <= 11; ++v) {
              const float d1 = fmaf((float)v, step[1], base[1]);
              const float m = fmaf(d1, fmaf(p.G[2], d1, u), t0);
              float w = ex2_approx(fmaf(m, kNegThirtyLog2e, l2n));
#pragma unroll
              for (int e = 0; e <= DEG; ++e) {
                S[e] += w;
                w *= d1;
              }
            }
            float pw = 1.f;
#pragma unroll
            for (int i = 0; i <= DEG; ++i) {
#pragma unroll
              for (int jx = 0; jx <= DEG - i; ++jx) M[mi(i, jx)] = fmaf(pw, S[jx], M[mi(i, jx)]);
              pw *= d0;
            }
          }
          scale = 100.f * step[0] * step[1] / 121.f;
        }
        const float R = I * scale * M[0];
        float al, be;
        if (in.mode == kModeInner) {
          al = c;
          be = 0.f;
          f = fmaf(c, R, f);
        } else if (in.mode == kModeL2Atom) {
          al = R - c;
          be = 1.f;
          f += R * (0.5f * R - c);
        } else {
          al = c;
          be = in.beta ? __ldg(in.beta + gi) : in.beta_const;
        }
        float A[NPSI];
        first_psi<K, NM>(M, p.G, A);
#pragma unroll
        for (int k = 0; k < NPSI; ++k) {
          A[k] *= scale;
          Sa[k] = fmaf(al, A[k], Sa[k]);
        }
        if constexpr (ORDER > 1) {
          float BC[NPSI][NPSI];
          psi_gram<K, true>(M, p.G, BC);
          const float as = al * scale;
#pragma unroll
          for (int k = 0; k < NPSI; ++k)
#pragma unroll
            for (int l = 0; l < NPSI; ++l) {
              Ta[k][l] = fmaf(as, BC[k][l], Ta[k][l]);
              Ub[k][l] = fmaf(be * A[k], A[l], Ub[k][l]);
            }
        }
      }
    }
    accumulate_pair<K, ORDER>(p, fr, I, Sa, Ta, Ub, gacc, hacc);
  }

  float vals_f = f;
  float gv[P];
#pragma unroll
  for (int i = 0; i < P; ++i) gv[i] = gacc[i].get();
  for (int off = cfg.ag; off < 32; off <<= 1) {
    vals_f += __shfl_xor_sync(0xffffffffu, vals_f, off);
#pragma unroll
    for (int i = 0; i < P; ++i) gv[i] += __shfl_xor_sync(0xffffffffu, gv[i], off);
    if constexpr (ORDER > 1) {
#pragma unroll
      for (int i = 0; i < NH; ++i) hacc[i] += __shfl_xor_sync(0xffffffffu, hacc[i], off);
    }
  }
  if (!valid || sub != 0) return;
  const size_t N = at.n;
  float *dst = part + (size_t)chunk * cfg.qn * N + j;
  dst[0] = vals_f;
#pragma unroll
  for (int i = 0; i < P; ++i) dst[(1 + i) * N] = gv[i];
  if constexpr (ORDER > 1) {
#pragma unroll
    for (int i = 0; i < NH; ++i) dst[(1 + P + i) * N] = hacc[i];
  }
}

// Sum chunk partials (FP64) in chunk order, expand the packed Hessian and
// apply the isotropic chain rule r_aniso = (s, .., s, 0, ..).  A block covers
// kFinAtoms atoms; thread t sums values q = t / kFinAtoms, + 32, ... of atom
// t % kFinAtoms (the loads of consecutive atoms share sectors), then all the
// block's threads write the atoms' outputs.  Few atoms per block spread the
// FP64 adds over many SMs' FP64 pipes (16 cycles per warp instruction each).
constexpr int kRedSlices = 8;
constexpr int kFinAtoms = 4;
constexpr int kFinThreads = 32 * kRedSlices;
// The body of one block of the finalize launch (the launch's block; a
// multi-problem launch maps its blocks to (problem, block)).
template <int K>
__device__ __forceinline__ void finalize_body(const float *part, const DerivCfg &cfg, int n,
                                              int deriv_order, int r_iso, const DerivOut &out,
                                              const double *f_extra, const int *order, int block) {
  constexpr int D = K + 1;
  constexpr int P = n_par<K>();
  constexpr int QN = 1 + P + P * (P + 1) / 2;
  // chunk sums in FP64 in chunk order: thread (atom, ty) sums values
  // q = ty, ty + 32, ... of its atom, all loads independent
  __shared__ double vs[QN][kFinAtoms];
  const int tx = threadIdx.x % kFinAtoms, ty = threadIdx.x / kFinAtoms;
  const int slot = block * kFinAtoms + tx;
  if (slot < n)
    for (int q = ty; q < cfg.qn; q += kFinThreads / kFinAtoms) {
      double t = 0.0;
#pragma unroll 4
      for (int c = 0; c < cfg.nchunks; ++c) t += (double)part[((size_t)c * cfg.qn + q) * n + slot];
      vs[q][tx] = t;
    }
  __syncthreads();
  // outputs of the block's atoms, written by all threads from the sums
  // (consecutive threads write consecutive entries of an atom's block)
  const int nb = min(kFinAtoms, n - (int)block * kFinAtoms);
  auto atom_of = [&](int t) {
    const int sl = block * kFinAtoms + t;
    return order ? order[sl] : sl;
  };
  // entry (a, b) of the full Hessian from the packed upper triangle
  auto hv = [&](int a, int b, int t) -> double {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    return vs[1 + P + lo * P - lo * (lo - 1) / 2 + (hi - lo)][t];
  };
  const double fx = f_extra ? f_extra[0] : 0.0;
  if (!r_iso) {
    for (int e = threadIdx.x; e < nb * (1 + P); e += blockDim.x) {
      const int t = e / (1 + P), q = e - t * (1 + P);
      const int j = atom_of(t);
      if (q == 0) out.f[j] = vs[0][t] + fx;
      else out.g[(size_t)j * P + q - 1] = vs[q][t];
    }
    if (deriv_order > 1)
      for (int e = threadIdx.x; e < nb * P * P; e += blockDim.x) {
        const int t = e / (P * P), ab = e - t * (P * P), a = ab / P, b = ab - a * P;
        out.H[(size_t)atom_of(t) * P * P + ab] = hv(a, b, t);
      }
    return;
  }
  // isotropic: parameters (I, x, s); s maps to the D diagonal r entries
  // (r_aniso = (s, .., s, 0, ..)), so its derivatives sum those entries'
  constexpr int PI = 2 + D;
  auto src = [](int a, int q) { return a < 1 + D ? a : 1 + D + q; };
  for (int e = threadIdx.x; e < nb * (1 + PI); e += blockDim.x) {
    const int t = e / (1 + PI), q = e - t * (1 + PI);
    const int j = atom_of(t);
    if (q == 0) {
      out.f[j] = vs[0][t] + fx;
    } else {
      const int a = q - 1;
      double gsum = 0.0;
      if (a <= D) {
        gsum = vs[1 + a][t];
      } else {
#pragma unroll
        for (int qq = 0; qq < D; ++qq) gsum += vs[1 + 1 + D + qq][t];
      }
      out.g[(size_t)j * PI + a] = gsum;
    }
  }
  if (deriv_order > 1)
    for (int e = threadIdx.x; e < nb * PI * PI; e += blockDim.x) {
      const int t = e / (PI * PI), ab = e - t * (PI * PI), a = ab / PI, b = ab - a * PI;
      const int na = a < 1 + D ? 1 : D, nbb = b < 1 + D ? 1 : D;
      double hs = 0.0;
      for (int qa = 0; qa < na; ++qa)
        for (int qb = 0; qb < nbb; ++qb) hs += hv(src(a, qa), src(b, qb), t);
      out.H[(size_t)atom_of(t) * PI * PI + ab] = hs;
    }
}

template <int K>
__global__ void __launch_bounds__(kFinThreads)
    gr_deriv_finalize_kernel(const float *part, DerivCfg cfg, int n, int deriv_order,
                             int r_iso, DerivOut out, const double *f_extra,
                             const int *order) {
  finalize_body<K>(part, cfg, n, deriv_order, r_iso, out, f_extra, order, blockIdx.x);
}

// 1/2 sum C^2 helper: block partial sums (FP32 compensated per thread, FP64
// across the block), then a fixed-order FP64 finalize.
__global__ void gr_sumsq_kernel(const float *C, size_t n, double *part) {
  __shared__ double sh[256];
  CAcc acc;
  acc.zero();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float c = C[i];
    acc.add(c * c);
  }
  sh[threadIdx.x] = (double)acc.s + (double)acc.c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void gr_sumsq_finalize_kernel(const double *part, int n, double scale,
                                         double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += part[i];
  out[0] = scale * s;
}

constexpr int kSumSqBlocks = 304;

int launch_sum_squares(const float *C, size_t n, double *out, void *ws,
                       size_t ws_bytes, cudaStream_t stream) {
  if (ws_bytes < align_up(kSumSqBlocks * sizeof(double))) return kErrWorkspace;
  double *part = static_cast<double *>(ws);
  gr_sumsq_kernel<<<kSumSqBlocks, 256, 0, stream>>>(C, n, part);
  gr_sumsq_finalize_kernel<<<1, 32, 0, stream>>>(part, kSumSqBlocks, 0.5, out);
  note_launches(2);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

Tuning g_tuning;

int tuning_set(Tuning &t, int key, int value) {
  if (key == 0 && value >= 32 && value <= (1 << 26)) {
    t.deriv_target_warps = value;
    return kOk;
  }
  if (key == 1 && value >= 1 && value <= 65536) {
    t.deriv_min_angles = value;
    return kOk;
  }
  if (key == 2 && (value == 0 || (value >= 1 && value <= 32 && (value & (value - 1)) == 0))) {
    t.deriv_atoms_per_warp = value;
    return kOk;
  }
  if (key == 3 && value >= 1 && value <= 3) {
    t.proj_form = value;
    return kOk;
  }
  if (key == 4 && value >= 0) {
    t.proj_split_cells = value;
    return kOk;
  }
  if (key == 6 && value >= 0) {
    t.deriv_split_lanes = value;
    return kOk;
  }
  if (key == 7 && value >= 0) {
    t.deriv_one_mb = value;
    return kOk;
  }
  if (key == 8 && (value == 0 || value == 1)) {
    t.deriv_wide_rows = value;
    return kOk;
  }
  if (key == 9 && (value == 1 || value == 4)) {
    t.deriv_block_warps = value;
    return kOk;
  }
  return kErrArg;
}

int tuning_get(const Tuning &t, int key) {
  return key == 0 ? t.deriv_target_warps : key == 1 ? t.deriv_min_angles
         : key == 2 ? t.deriv_atoms_per_warp : key == 3 ? t.proj_form
         : key == 4 ? t.proj_split_cells
         : key == 6 ? t.deriv_split_lanes : key == 7 ? t.deriv_one_mb
         : key == 8 ? t.deriv_wide_rows : key == 9 ? t.deriv_block_warps : -1;
}

size_t derivs_workspace_bytes(int K, int n_atoms, int n_angles, int order, const Tuning &t) {
  DerivCfg c = deriv_cfg(K, n_atoms, n_angles, order, t);
  size_t b = align_up((size_t)c.nchunks * c.qn * (size_t)n_atoms * sizeof(float));
  b += align_up(kSumSqBlocks * sizeof(double)) + align_up(sizeof(double));
  return b;
}

int launch_derivs(const Atoms &at, const Geom &g, const DerivIn &in,
                  const DerivOut &out, void *ws, size_t ws_bytes,
                  cudaStream_t stream, const Tuning &t) {
  const int K = g.K;
  if (at.n <= 0) return kOk;
  if (in.order < 1 || in.order > 2) return kErrArg;
  // the pixel-integrated kernel walks whole pairs per lane (no cell split);
  // its chunking never needs more workspace than the split one
  DerivCfg c = deriv_cfg(K, at.n, g.n_angles, in.order, t, !in.psf);
  if (ws == nullptr || ws_bytes < derivs_workspace_bytes(K, at.n, g.n_angles, in.order, t))
    return kErrWorkspace;
  char *wp = static_cast<char *>(ws);
  float *part = reinterpret_cast<float *>(wp);
  wp += align_up((size_t)c.nchunks * c.qn * (size_t)at.n * sizeof(float));
  double *sumsq_part = reinterpret_cast<double *>(wp);
  wp += align_up(kSumSqBlocks * sizeof(double));
  double *f_extra = reinterpret_cast<double *>(wp);
  const double *fe = nullptr;
  if (in.mode == kModeL2Atom) {
    const size_t cells = (size_t)g.n_angles * g.ax[0].n * (K == 2 ? g.ax[1].n : 1);
    int rc = launch_sum_squares(in.alpha, cells, f_extra, sumsq_part,
                                align_up(kSumSqBlocks * sizeof(double)), stream);
    if (rc != kOk) return rc;
    fe = f_extra;
  }
  const int warps = ((at.n + c.ag - 1) / c.ag) * c.nchunks;
  const int blocks = (warps + 3) / 4;
  const float s = 0.5f / g.ax[0].inv_step;  // cell half-width (pixel-integrated operator)
  // one-warp blocks (Tuning key 9) for the kernels with one angle per lane
  const bool bw1 = t.deriv_block_warps == 1;
  const int blocks1 = warps;
  timer_mark(2, 0, stream);
  if (in.psf) {
    if (K == 1) {
      if (in.order == 1) gr_psf_deriv_kernel<1, 1><<<blocks, 128, 0, stream>>>(at, g, in, c, part, s);
      else gr_psf_deriv_kernel<1, 2><<<blocks, 128, 0, stream>>>(at, g, in, c, part, s);
    } else {
      if (in.order == 1) gr_psf_deriv_kernel<2, 1><<<blocks, 128, 0, stream>>>(at, g, in, c, part, s);
      else gr_psf_deriv_kernel<2, 2><<<blocks, 128, 0, stream>>>(at, g, in, c, part, s);
    }
  } else {
    // at most one angle per lane: a lane's angles a_lo + sub + k sg lie
    // below a_lo + ch
    const bool one = c.ch <= c.sg / c.rs;
    const bool wide = t.deriv_wide_rows != 0;
    if (K == 1) {
      if (in.order == 1) {
        if (one) gr_deriv_kernel<1, 1, true><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
        else gr_deriv_kernel<1, 1, false><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
      } else {
        if (one && bw1)
          gr_deriv_kernel<1, 2, true, false, 1><<<blocks1, 32, 0, stream>>>(at, g, in, c, part);
        else if (one) gr_deriv_kernel<1, 2, true><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
        else gr_deriv_kernel<1, 2, false><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
      }
    } else {
      if (in.order == 1) {
        if (one && bw1)
          gr_deriv_kernel<2, 1, true, false, 1><<<blocks1, 32, 0, stream>>>(at, g, in, c, part);
        else if (one) gr_deriv_kernel<2, 1, true><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
        else gr_deriv_kernel<2, 1, false><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
      } else if (wide) {
        if (one && bw1)
          gr_deriv_kernel<2, 2, true, true, 1><<<blocks1, 32, 0, stream>>>(at, g, in, c, part);
        else if (one)
          gr_deriv_kernel<2, 2, true, true><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
        else gr_deriv_kernel<2, 2, false, true><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
      } else {
        if (one && bw1)
          gr_deriv_kernel<2, 2, true, false, 1><<<blocks1, 32, 0, stream>>>(at, g, in, c, part);
        else if (one) gr_deriv_kernel<2, 2, true><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
        else gr_deriv_kernel<2, 2, false><<<blocks, 128, 0, stream>>>(at, g, in, c, part);
      }
    }
  }
  timer_mark(2, 1, stream);
  const int fblocks = (at.n + kFinAtoms - 1) / kFinAtoms;
  if (K == 1)
    gr_deriv_finalize_kernel<1><<<fblocks, kFinThreads, 0, stream>>>(
        part, c, at.n, in.order, at.r_iso, out, fe, at.order);
  else
    gr_deriv_finalize_kernel<2><<<fblocks, kFinThreads, 0, stream>>>(
        part, c, at.n, in.order, at.r_iso, out, fe, at.order);
  note_launches(2);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

// ---- multi-problem launches (2D Hessians, one angle per lane) ------------
// The derivatives of a problem run only on its first iteration or after an
// accepted trial (a rejected trial leaves its atoms and fields unchanged),
// and not once its fit has stopped.
__device__ __forceinline__ bool batch_derivs_wanted(const BatchProb &B, int active) {
  if (!active) return false;
  const int c = *B.counter;
  return !(c > 0 && c <= B.hist_len && !B.hist_acc[c - 1]);
}

__global__ void __launch_bounds__(128, GR_HESS2D_MIN_BLOCKS)
    gr_batch_deriv_kernel(const BatchProb *__restrict__ probs, const int *__restrict__ off,
                          int n, const int *__restrict__ active) {
  const int p = batch_find(off, n, blockIdx.x);
  const BatchProb &B = probs[p];
  if (!batch_derivs_wanted(B, active[p])) return;
  deriv_body<1, 2, true>(B.cur, B.g, B.din, B.cfg, B.part, ((int)blockIdx.x - off[p]) * 4);
}

__global__ void __launch_bounds__(kFinThreads)
    gr_batch_finalize_kernel(const BatchProb *__restrict__ probs, const int *__restrict__ off,
                             int n, const int *__restrict__ active) {
  const int p = batch_find(off, n, blockIdx.x);
  const BatchProb &B = probs[p];
  if (!batch_derivs_wanted(B, active[p])) return;
  finalize_body<1>(B.part, B.cfg, B.cur.n, 2, B.cur.r_iso, B.dout, nullptr, nullptr,
                   blockIdx.x - off[p]);
}

int finalize_blocks(int n_atoms) { return (n_atoms + kFinAtoms - 1) / kFinAtoms; }

int launch_batch_derivs(const BatchLaunch &b, cudaStream_t stream) {
  if (b.grid_deriv <= 0) return kOk;
  gr_batch_deriv_kernel<<<b.grid_deriv, 128, 0, stream>>>(b.probs, b.off_deriv, b.n, b.active);
  gr_batch_finalize_kernel<<<b.grid_fin, kFinThreads, 0, stream>>>(b.probs, b.off_fin, b.n,
                                                                   b.active);
  note_launches(2);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int preload_derivs() {
  return preload_fn(gr_deriv_kernel<1, 1, false>) + preload_fn(gr_deriv_kernel<1, 2, false>) +
         preload_fn(gr_deriv_kernel<2, 1, false>) + preload_fn(gr_deriv_kernel<2, 2, false>) +
         preload_fn(gr_deriv_kernel<1, 1, true>) + preload_fn(gr_deriv_kernel<1, 2, true>) +
         preload_fn(gr_deriv_kernel<2, 1, true>) + preload_fn(gr_deriv_kernel<2, 2, true>) +
         preload_fn(gr_deriv_kernel<2, 2, false, true>) +
         preload_fn(gr_deriv_kernel<2, 2, true, true>) +
         preload_fn(gr_deriv_kernel<1, 2, true, false, 1>) +
         preload_fn(gr_deriv_kernel<2, 1, true, false, 1>) +
         preload_fn(gr_deriv_kernel<2, 2, true, false, 1>) +
         preload_fn(gr_deriv_kernel<2, 2, true, true, 1>) +
         preload_fn(gr_psf_deriv_kernel<1, 1>) + preload_fn(gr_psf_deriv_kernel<1, 2>) +
         preload_fn(gr_psf_deriv_kernel<2, 1>) + preload_fn(gr_psf_deriv_kernel<2, 2>) +
         preload_fn(gr_deriv_finalize_kernel<1>) + preload_fn(gr_deriv_finalize_kernel<2>) +
         preload_fn(gr_sumsq_kernel) + preload_fn(gr_sumsq_finalize_kernel) +
         preload_fn(gr_batch_deriv_kernel) + preload_fn(gr_batch_finalize_kernel);
}

}  // namespace gr
