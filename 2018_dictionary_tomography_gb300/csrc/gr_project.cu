// Forward projection of Gaussian atoms (sm_103a).
//
// Replaces the reference's dense per-cell loops __RadProj
// (GaussDictCode/bin/NewtonBases2D.py:286-296) and __RadProj_3D/_2p5D
// (GaussDictCode/bin/NewtonBases.py:731-756), which evaluate every atom at
// every detector cell.  Here:
//   1. gr_bin_kernel: per (atom, angle) pair, compute the support box of
//      m <= 1 and set the atom's bit in the bitmap of every detector tile the
//      box touches (integer atomicOr, so the bitmap does not depend on the
//      order in which pairs run).
//   2. gr_project3d_kernel (3D / 2.5D detectors) and gr_project1d_kernel
//      (2D sinograms): one warp per (angle, tile) item.  The warp meets the
//      tile's atoms in increasing index order and sums every cell over its
//      atoms in that order with a compensated add and no float atomics, so
//      results are bitwise reproducible.  The epilogue writes the sinogram
//      and, fused, the residual or KL weight fields and per-tile loss
//      partials.  The 3D kernel is persistent: warps take items from a
//      counter, so tiles of uneven weight do not leave warps idle.
//   3. gr_loss_finalize_kernel: fixed-order FP64 sum of the loss partials.
#include "gr_kernels.cuh"

namespace gr {

// pairs (2D only, nullable): the pair's projection data as the 2D
// projection stages it, two float4 per (angle, atom) at [a n + j], written
// here once instead of being recomputed by every tile the atom touches
// The body of a 128-thread block of the binning launch: atoms bx * 128 ..,
// angle a (the launch's block (bx, a); a multi-problem launch maps its
// blocks to (problem, bx, a)).
// flag, list, n_list (3D, nullable): the items some atom meets, listed once
// each (in no fixed order: the order changes no result) for a forward that
// skips the others.  Only the first bit set in a word can be an item's first,
// so an item's flag is tested once per word it uses, not once per atom.
template <int K>
__device__ __forceinline__ void bin_body(const Atoms &at, const Geom &g, const TileCfg &tc,
                                         uint32_t *bitmap, int W, float4 *pairs, int bx,
                                         int a, uint32_t *flag = nullptr, int *list = nullptr,
                                         int *n_list = nullptr) {
  const int j = bx * 128 + (int)threadIdx.x;
  const uint32_t bit = 1u << (j & 31);
  const size_t base = (size_t)a * tc.ntiles;
  const int wj = j >> 5;
  if constexpr (K == 1) {
    // a warp holds 32 consecutive atoms: one bitmap word per tile.  Their
    // bits are merged per tile across the warp (one atomicOr per tile the
    // warp touches, not one per atom and tile: the 32 atoms of a word would
    // otherwise all hit the same address)
    int t_lo = 1 << 30, t_hi = -1;
    if (j < at.n) {
      Frame<1> f;
      load_frame<1>(g.frames, a, f);
      Pair<1> p;
      pair_setup<1>(at, j, f, g, p);
      if (pairs) {
        float4 *rec = pairs + ((size_t)a * at.n + j) * 2;
        rec[0] = make_float4(p.qh[0], p.ql[0], p.G[0], p.l2amp);
        rec[1] = make_float4(__int_as_float(p.lo[0]), __int_as_float(p.hi[0]), p.sgn, 0.f);
      }
      if (p.lo[0] <= p.hi[0]) {
        t_lo = p.lo[0] / tc.t0;
        t_hi = p.hi[0] / tc.t0;
      }
    }
    const int w_lo = __reduce_min_sync(0xffffffffu, t_lo);
    const int w_hi = __reduce_max_sync(0xffffffffu, t_hi);
    for (int t = w_lo; t <= w_hi; ++t) {
      const unsigned bits = __reduce_or_sync(0xffffffffu, (t >= t_lo && t <= t_hi) ? bit : 0u);
      if ((threadIdx.x & 31) == 0 && bits) atomicOr(bitmap + (base + t) * W + wj, bits);
    }
  } else {
    if (j >= at.n) return;
    Frame<K> f;
    load_frame<K>(g.frames, a, f);
    Pair<K> p;
    pair_setup<K>(at, j, f, g, p);
    if (p.lo[0] > p.hi[0]) return;
    if (p.lo[1] > p.hi[1]) return;
    const int r_lo = p.lo[0] / tc.t0, r_hi = p.hi[0] / tc.t0;
    const int c_lo = p.lo[1] / tc.t1, c_hi = p.hi[1] / tc.t1;
    for (int tr = r_lo; tr <= r_hi; ++tr)
      for (int tcix = c_lo; tcix <= c_hi; ++tcix) {
        const size_t item = base + (size_t)tr * tc.nt1 + tcix;
        if (flag == nullptr) {
          atomicOr(bitmap + item * W + wj, bit);
        } else if (atomicOr(bitmap + item * W + wj, bit) == 0u &&
                   atomicExch(flag + item, 1u) == 0u) {
          list[atomicAdd(n_list, 1)] = (int)item;
        }
      }
  }
}

template <int K>
__global__ void __launch_bounds__(128) gr_bin_kernel(Atoms at, Geom g,
                                                     TileCfg tc, uint32_t *bitmap,
                                                     int W, float4 *pairs, uint32_t *flag,
                                                     int *list, int *n_list) {
  bin_body<K>(at, g, tc, bitmap, W, pairs, blockIdx.x, blockIdx.y, flag, list, n_list);
}

// Per-cell KL term f log(f/g) - f + g = g h(u), u = f/g, h(u) = u log u - u + 1,
// evaluated without cancellation: a series in e = u - 1 near u = 1.
__device__ __forceinline__ float kl_term(float f, float g) {
  if (!(f > 0.f)) return g;
  const float e = (f - g) / g;
  float h;
  if (fabsf(e) < 0.125f) {
    // h = sum_{k>=2} (-1)^k e^k / (k (k-1))
    float e2 = e * e;
    h = e2 * (0.5f + e * (-1.f / 6.f + e * (1.f / 12.f + e * (-1.f / 20.f +
             e * (1.f / 30.f + e * (-1.f / 42.f + e * (1.f / 56.f)))))));
  } else {
    const float u = f / g;
    h = u * logf(u) - u + 1.f;
  }
  return g * h;
}

// 3D detectors: a warp per (angle, tile) item.  Its atoms come from the
// tile's bitmap in increasing index order; the pair data of each batch of 32
// atoms is computed in parallel (one atom per lane) and staged in shared
// memory (three float4 per atom, read as broadcasts, the tile-local clipped
// box packed in one word); then each atom is evaluated densely over its box,
// lanes spread over the box cells, into shared-memory cell sums with a
// compensated (Kahan/Neumaier) add.  Each cell therefore sums its atoms in
// atom-index order, with no float atomics: results are bitwise reproducible.
// Sums and compensations use a padded row stride S so that the cells of one
// box row-block fall in different banks.  Tiles are ROWS x 32 cells.
template <int ROWS, int S>
struct Proj3Smem {
  static constexpr int kAcc = ROWS * S;
  static constexpr int kRing = 128;     // ring list of atom indices
  static constexpr int kFloats = 2 * kAcc + 32 * 12 + ROWS + 32 + kRing;
};

// NW = 1: persistent warps, each (angle, tile) item walked by one warp.
// NW = kProjWarps: persistent blocks, each item walked by the whole block,
// warp w taking the atoms of bitmap words [w wq, (w + 1) wq), wq = ceil(W/NW),
// into its own cell sums; the block then combines the warps' sums per cell
// in warp order (compensated).  The word ranges depend on W only, so every
// tiling still gives the same cell sums.  Used when a problem has too few
// items to keep the SMs busy: the slowest item, not the total, then sets
// the kernel time, and splitting its atom list cuts that item's latency.
// With loss_out, the last block (or warp) to finish sums the items' loss
// partials in item order (no separate finalize launch).
// LIST: take only the n_list[0] items of item_list (those some atom meets;
// the loss partials of the others are already in place).  A template
// parameter, so that the forward of every item keeps its own registers.
template <int ROWS, int S, int NW, bool LIST>
__global__ void __launch_bounds__(kProjWarps * 32)
    gr_project3d_kernel(Atoms at, Geom g, TileCfg tc, const uint32_t *bitmap, int W,
                        ProjOut out, int *next_item, double *loss_out,
                        const int *item_list, const int *n_list) {
  static_assert(NW == 1 || NW == kProjWarps, "a split item takes the whole block");
  using L = Proj3Smem<ROWS, S>;
  constexpr int kRing = L::kRing;
  static_assert((kRing & (kRing - 1)) == 0 && kRing >= 64, "ring");
  extern __shared__ float smem[];
  __shared__ int s_item;
  __shared__ double s_loss[NW];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_items = g.n_angles * tc.ntiles;
  const int n_take = LIST ? *n_list : n_items;
  float *acc = smem + (size_t)warp * L::kFloats;
  float *cmp = acc + L::kAcc;
  float4 *prm = reinterpret_cast<float4 *>(cmp + L::kAcc);  // 16-byte aligned
  float *pc0 = reinterpret_cast<float *>(prm + 32 * 3);
  float *pc1 = pc0 + ROWS;
  int *list = reinterpret_cast<int *>(pc1 + 32);
  const int wq = (W + NW - 1) / NW;
  const int w_lo = min(W, warp * wq * (NW > 1)), w_hi = NW > 1 ? min(W, w_lo + wq) : W;

  // persistent warps (blocks): each takes the next (angle, tile) item from a
  // counter, so heavy tiles do not hold the others idle; what an item
  // computes does not depend on which warp (block) takes it
  for (;;) {
  int item = 0;
  if constexpr (NW == 1) {
    if (lane == 0) item = atomicAdd(next_item, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= n_take) break;  // whole warp leaves together
    __syncwarp();  // the previous item's epilogue reads are done
  } else {
    if (threadIdx.x == 0) s_item = atomicAdd(next_item, 1);
    __syncthreads();
    item = s_item;
    if (item >= n_take) break;  // whole block leaves together
  }
  if constexpr (LIST) item = item_list[item];
  const int a = item / tc.ntiles, t = item - a * tc.ntiles;
  const int tr = t / tc.nt1, tcix = t - tr * tc.nt1;
  const int r0 = tr * ROWS, c0 = tcix * 32;
  const int D0 = g.ax[0].n, D1 = g.ax[1].n;

  for (int e = lane; e < L::kAcc; e += 32) {
    acc[e] = 0.f;
    cmp[e] = 0.f;
  }
  for (int e = lane; e < ROWS; e += 32)
    pc0[e] = (r0 + e < D0) ? g.ax[0].coords[r0 + e] : 0.f;
  pc1[lane] = (c0 + lane < D1) ? g.ax[1].coords[c0 + lane] : 0.f;
  Frame<2> f;
  load_frame<2>(g.frames, a, f);
  __syncwarp();

  // The warp's atoms of the tile, in index order, pass through a ring list:
  // a refill reads 32 bitmap words (one per lane) and appends the atoms of as
  // many whole words as fit, so every batch but the last holds 32 atoms
  // however sparse the bitmap is.
  const uint32_t *words = bitmap + (size_t)item * W;
  int head = 0, count = 0, wb = w_lo;
  while (true) {
    while (count < 32 && wb < w_hi) {
      const int wi = wb + lane;
      uint32_t wd = wi < w_hi ? words[wi] : 0u;
      const int cnt = __popc(wd);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      // incl never decreases along the lanes, so the lanes that fit are a
      // prefix; at least one word fits (count < 32, a word adds <= 32)
      const bool take = incl <= kRing - count;
      const unsigned tmask = __ballot_sync(0xffffffffu, take);
      const int ntake = __popc(tmask);
      if (take) {
        int pos = head + count + incl - cnt;
        while (wd) {
          const int b = __ffs(wd) - 1;
          list[(pos++) & (kRing - 1)] = (wi << 5) + b;
          wd &= wd - 1;
        }
      }
      count += __shfl_sync(0xffffffffu, incl, ntake - 1);
      wb += ntake;
      __syncwarp();
    }
    if (count == 0) break;
    {
      __syncwarp();  // every lane is done with the previous batch's data
      const int nb = min(32, count);
      // C.y: the tile-local clipped box as first row | first column << 8 |
      // width << 16 | rows << 24 (0: empty), C.z: 1 / width; both formed
      // here, one atom per lane, rather than by the whole warp per atom
      float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, C = A;
      if (lane < nb) {
        Pair<2> p;
        pair_setup<2>(at, list[(head + lane) & (kRing - 1)], f, g, p);
        const int lr0 = max(p.lo[0], r0) - r0, lr1 = min(p.hi[0], r0 + ROWS - 1) - r0;
        const int lc0 = max(p.lo[1], c0) - c0, lc1 = min(p.hi[1], c0 + 31) - c0;
        const bool empty = lr0 > lr1 || lc0 > lc1;
        A = make_float4(p.qh[0], p.ql[0], p.qh[1], p.ql[1]);
        B = make_float4(p.G[0], 2.f * p.G[1], p.G[2], p.l2amp);
        C.x = p.sgn;
        const int bw = lc1 - lc0 + 1;
        C.y = __uint_as_float(empty ? 0u
                                    : (unsigned)(lr0 | (lc0 << 8) | (bw << 16) |
                                                 ((lr1 - lr0 + 1) << 24)));
        C.z = empty ? 0.f : __frcp_rn((float)bw);
      }
      head += nb;
      count -= nb;
      prm[lane * 3 + 0] = A;
      prm[lane * 3 + 1] = B;
      prm[lane * 3 + 2] = C;
      __syncwarp();
      for (int sI = 0; sI < nb; ++sI) {
        const float4 qC = prm[sI * 3 + 2];
        const unsigned box = __float_as_uint(qC.y);
        if (box == 0u) continue;  // warp-uniform
        const int lr0 = box & 0xff, lc0 = (box >> 8) & 0xff, bw = (box >> 16) & 0xff;
        const int ncell = (int)(box >> 24) * bw;
        const float inv_bw = qC.z;
        const float4 qA = prm[sI * 3 + 0], qB = prm[sI * 3 + 1];
        for (int e = lane; e < ncell; e += 32) {
          // (e + 1/2) / bw is at least 1/(2 bw) from an integer, far more
          // than the rounding of the product: the row index is exact
          const int rr = (int)(((float)e + 0.5f) * inv_bw);
          const int lr = lr0 + rr;
          const int lc = lc0 + (e - rr * bw);
          const float d0 = (pc0[lr] - qA.x) - qA.y;
          const float d1 = (pc1[lc] - qA.z) - qA.w;
          const float m = fmaf(d0, fmaf(qB.x, d0, qB.y * d1), qB.z * d1 * d1);
          if (m <= 1.f) {
            const float v = qC.x * ex2_approx(fmaf(m, kNegThirtyLog2e, qB.w));
            const int ci = lr * S + lc;
            const float s0 = acc[ci];
            const float tt = s0 + v;
            cmp[ci] += (fabsf(s0) >= fabsf(v)) ? ((s0 - tt) + v) : ((v - tt) + s0);
            acc[ci] = tt;
          }
        }
        __syncwarp();
      }
    }
  }
  if constexpr (NW == 1) __syncwarp();
  else __syncthreads();

  // epilogue: write the tile, fused fit fields and loss partial; a split
  // item's cells combine the warps' sums in warp order
  // The data values of a batch of a thread's cells are loaded before any of
  // them is written (the output fields may alias nothing, but the compiler
  // cannot know that), so a batch costs one memory latency, not one per cell.
  constexpr int kPer = ROWS / NW;                 // cells per thread
  constexpr int kBatch = kPer < (NW == 1 ? 8 : 4) ? kPer : (NW == 1 ? 8 : 4);
  static_assert(kPer % kBatch == 0, "batch");
  const bool want_data = out.epilogue == kEpiL2 || out.epilogue == kEpiKL;
  const int e0 = NW == 1 ? lane : (int)threadIdx.x;
  const int col = c0 + lane;
  float lsum = 0.f, lcmp = 0.f;
  for (int eb = 0; eb < kPer; eb += kBatch) {
    float dv[kBatch];
#pragma unroll
    for (int i = 0; i < kBatch; ++i) {
      const int row = r0 + ((e0 + (eb + i) * NW * 32) >> 5);
      dv[i] = (want_data && row < D0 && col < D1)
                  ? __ldg(out.data + ((size_t)a * D0 + row) * D1 + col)
                  : 0.f;
    }
#pragma unroll
    for (int i = 0; i < kBatch; ++i) {
    const int lr = (e0 + (eb + i) * NW * 32) >> 5;
    const int row = r0 + lr;
    if (row >= D0 || col >= D1) continue;
    const int ci = lr * S + lane;
    float v;
    if constexpr (NW == 1) {
      v = acc[ci] + cmp[ci];
    } else {
      float s0 = 0.f, c0s = 0.f;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const float *aw = smem + (size_t)w * L::kFloats;
        const float x = aw[ci] + aw[L::kAcc + ci];
        const float tt = s0 + x;
        c0s += (fabsf(s0) >= fabsf(x)) ? ((s0 - tt) + x) : ((x - tt) + s0);
        s0 = tt;
      }
      v = s0 + c0s;
    }
    const size_t gi = ((size_t)a * D0 + row) * D1 + col;
    if (out.R) out.R[gi] = v;
    float l = 0.f;
    if (out.epilogue == kEpiL2) {
      const float res = v - dv[i];
      if (out.alpha) out.alpha[gi] = res;
      l = 0.5f * res * res;
    } else if (out.epilogue == kEpiKL) {
      const float fo = dv[i];
      const float gg = v + out.bg;
      const float ig = 1.f / gg;
      if (out.alpha) out.alpha[gi] = 1.f - fo * ig;
      if (out.beta) out.beta[gi] = fo * ig * ig;
      l = kl_term(fo, gg);
    }
    const float tt = lsum + l;
    lcmp += (fabsf(lsum) >= fabsf(l)) ? ((lsum - tt) + l) : ((l - tt) + lsum);
    lsum = tt;
    }
  }
  if (out.loss_part) {
    double d = warp_sum_d((double)lsum + (double)lcmp);
    if constexpr (NW == 1) {
      if (lane == 0) out.loss_part[item] = d;
    } else {
      if (lane == 0) s_loss[warp] = d;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tl = 0.0;
#pragma unroll
        for (int w = 0; w < NW; ++w) tl += s_loss[w];
        out.loss_part[item] = tl;
      }
    }
  }
  if constexpr (NW > 1) __syncthreads();  // cell sums and s_item are reused
  }

  if (loss_out && out.loss_part) {
    // the last warp (block) to finish sums the items' partials in item order
    const int units = NW == 1 ? (int)gridDim.x * kProjWarps : (int)gridDim.x;
    if (NW > 1 && warp != 0) return;
    int last = 0;
    if (lane == 0) {
      __threadfence();
      last = atomicAdd(next_item + 1, 1) == units - 1;
    }
    if (__shfl_sync(0xffffffffu, last, 0)) {
      __threadfence();
      sum_partials_warp(out.loss_part, n_items, loss_out, lane);
    }
  }
}

// 2D sinograms: atom footprints are a few cells wide, so a block owns a tile
// of 32 CPL consecutive cells of one angle, CPL cells per lane of every warp
// (lane l: cells l, l + 32, ...).  CPL = 2 (Tuning key 3, form 2) halves the
// tiles an atom of a wide footprint touches, and with them the listing,
// staging and binning per evaluated cell; narrow footprints leave more lanes
// idle in it.  The
// tile's atoms come from its bitmap in index order, in passes: a pass lists
// as many whole bitmap words as fit in NW*32 entries (block-wide prefix sum
// of the words' bit counts), every thread sets up the pair data of one listed
// atom in shared memory, and warp w adds the atoms of the w-th of NW
// contiguous slices of the pass's list to its lane's cell, in list order, in
// registers (compensated).  The warps' partial sums are combined in warp
// order: results depend only on the atoms listed, bitwise reproducible.
// LM: a pass lists up to LM * NW * 32 atoms (each thread stages LM of them),
// so tiles crossed by many atoms take fewer passes and barriers (2150 atoms x
// 153 angles: 87.9 us with one atom per thread, 82.6 with two, 79.5 with
// four; 512 atoms: 20.6, 20.7, 21.1 us)
// The body of one block of the 2D projection: (angle, tile) item of n_items
// (the launch's block; a multi-problem launch maps its blocks to (problem,
// item)).
template <bool KAHAN, int NW, int CPL = 1, int LM = 1>
__device__ __forceinline__ void project1d_body(const Atoms &at, const Geom &g, const TileCfg &tc,
                                               const uint32_t *bitmap, int W, const ProjOut &out,
                                               double *loss_out, int *done,
                                               const float4 *__restrict__ pairs, int item,
                                               int n_items) {
  constexpr int T = NW * 32;
  constexpr int LT = LM * T;
  __shared__ float4 prm[LT][2];
  __shared__ int list[LT];
  __shared__ int wsum[NW];
  __shared__ float parts[NW][2][32 * CPL];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = item / tc.ntiles, t = item - a * tc.ntiles;
  const int D0 = g.ax[0].n;
  int cell[CPL];
  float pc[CPL], acc[CPL], cmp[CPL];
#pragma unroll
  for (int k = 0; k < CPL; ++k) {
    cell[k] = t * tc.t0 + lane + 32 * k;
    pc[k] = cell[k] < D0 ? g.ax[0].coords[cell[k]] : 0.f;
    acc[k] = 0.f;
    cmp[k] = 0.f;
  }
  const float4 *apairs = pairs + (size_t)a * at.n * 2;

  const uint32_t *words = bitmap + (size_t)item * W;
  for (int wb = 0; wb < W;) {
    // thread k holds word wb + k; inclusive prefix of the bit counts
    const int wi = wb + (int)threadIdx.x;
    uint32_t wd = wi < W ? words[wi] : 0u;
    const int cnt = __popc(wd);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < NW; ++w)
      if (w < warp) incl += wsum[w];
    // the words that fit form a prefix (incl never decreases); one word
    // always fits (a word holds at most 32 <= LT atoms)
    const bool take = incl <= LT;
    const int pos = incl - cnt;
    if (take)
      for (int p = pos; wd; ++p) {
        list[p] = (wi << 5) + (__ffs(wd) - 1);
        wd &= wd - 1;
      }
    const int ntake = __syncthreads_count(take && wi < W);
    // entries listed: the inclusive count of the last word taken
    int total = 0;
    if (ntake > 0 && (int)threadIdx.x == ntake - 1) wsum[0] = incl;
    __syncthreads();
    total = wsum[0];
    wb += ntake > 0 ? ntake : W;   // ntake = 0 only past the last word
    // pair data of the listed atoms (set up once per pair by the binning
    // launch), up to LM per thread
    for (int e = threadIdx.x; e < total; e += T) {
      const float4 *rec = apairs + (size_t)list[e] * 2;
      prm[e][0] = __ldg(rec);
      prm[e][1] = __ldg(rec + 1);
    }
    __syncthreads();
    // warp w: slice [w total / NW, (w + 1) total / NW) in list order
    const int s_lo = (warp * total) / NW, s_hi = ((warp + 1) * total) / NW;
#pragma unroll 4
    for (int s2 = s_lo; s2 < s_hi; ++s2) {
      const float4 q0 = prm[s2][0];
      const float4 q1 = prm[s2][1];
      const int lo = __float_as_int(q1.x), hi = __float_as_int(q1.y);
#pragma unroll
      for (int k = 0; k < CPL; ++k) {
        if (cell[k] >= lo && cell[k] <= hi) {
          const float d = (pc[k] - q0.x) - q0.y;
          const float m = q0.z * d * d;
          if (m <= 1.f) {
            const float v = q1.z * ex2_approx(fmaf(m, kNegThirtyLog2e, q0.w));
            if (KAHAN) {
              const float tt = acc[k] + v;
              cmp[k] += (fabsf(acc[k]) >= fabsf(v)) ? ((acc[k] - tt) + v) : ((v - tt) + acc[k]);
              acc[k] = tt;
            } else {
              acc[k] += v;
            }
          }
        }
      }
    }
    __syncthreads();  // list, prm and wsum are reused by the next pass
  }
#pragma unroll
  for (int k = 0; k < CPL; ++k) {
    parts[warp][0][lane + 32 * k] = acc[k];
    parts[warp][1][lane + 32 * k] = cmp[k];
  }
  __syncthreads();
  __shared__ int s_last;
  if (warp == 0) {
    // combine the warps' partial sums in warp order (compensated)
    float l = 0.f;
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
      float s0 = 0.f, c0 = 0.f;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float v = parts[w][h][lane + 32 * k];
          const float tt = s0 + v;
          c0 += (fabsf(s0) >= fabsf(v)) ? ((s0 - tt) + v) : ((v - tt) + s0);
          s0 = tt;
        }
      }
      if (cell[k] < D0) {
        const float v = s0 + c0;
        const size_t gi = (size_t)a * D0 + cell[k];
        float lk = 0.f;
        if (out.R) out.R[gi] = v;
        if (out.epilogue == kEpiL2) {
          const float res = v - out.data[gi];
          if (out.alpha) out.alpha[gi] = res;
          lk = 0.5f * res * res;
        } else if (out.epilogue == kEpiKL) {
          const float fo = out.data[gi];
          const float gg = v + out.bg;
          const float ig = 1.f / gg;
          if (out.alpha) out.alpha[gi] = 1.f - fo * ig;
          if (out.beta) out.beta[gi] = fo * ig * ig;
          lk = kl_term(fo, gg);
        }
        l += lk;
      }
    }
    if (out.loss_part) {
      const double d = warp_sum_d((double)l);
      if (lane == 0) out.loss_part[item] = d;
      if (loss_out && lane == 0) {
        __threadfence();
        s_last = atomicAdd(done, 1) == n_items - 1;
      }
    }
  }  // warp 0
  if (!out.loss_part || !loss_out) return;
  __syncthreads();
  if (!s_last) return;
  // the last block to finish sums the per-tile partials, all its threads
  __threadfence();
  sum_partials_block<NW>(out.loss_part, n_items, loss_out);
}

template <bool KAHAN, int NW, int CPL = 1, int LM = 1>
__global__ void __launch_bounds__(NW * 32)
    gr_project1d_kernel(Atoms at, Geom g, TileCfg tc, const uint32_t *bitmap,
                        int W, ProjOut out, double *loss_out, int *done,
                        const float4 *__restrict__ pairs) {
  project1d_body<KAHAN, NW, CPL, LM>(at, g, tc, bitmap, W, out, loss_out, done, pairs,
                                     blockIdx.x, gridDim.x);
}

// ---- pixel-integrated operator: binning and projection -------------------
template <int K>
__global__ void __launch_bounds__(128) gr_psf_bin_kernel(Atoms at, Geom g, TileCfg tc,
                                                         uint32_t *bitmap, int W, float s) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (j >= at.n) return;
  Frame<K> f;
  load_frame<K>(g.frames, a, f);
  Pair<K> p;
  const bool ok = pair_setup<K>(at, j, f, g, p);
  PsfPair<K> q;
  psf_setup<K>(at, j, g, p, ok, s, q);
  if (q.lo[0] > q.hi[0]) return;
  const uint32_t bit = 1u << (j & 31);
  const size_t base = (size_t)a * tc.ntiles;
  const int wj = j >> 5;
  if constexpr (K == 1) {
    for (int t = q.lo[0] / tc.t0; t <= q.hi[0] / tc.t0; ++t)
      atomicOr(bitmap + (base + t) * W + wj, bit);
  } else {
    if (q.lo[1] > q.hi[1]) return;
    for (int tr = q.lo[0] / tc.t0; tr <= q.hi[0] / tc.t0; ++tr)
      for (int tcix = q.lo[1] / tc.t1; tcix <= q.hi[1] / tc.t1; ++tcix)
        atomicOr(bitmap + (base + (size_t)tr * tc.nt1 + tcix) * W + wj, bit);
  }
}

struct PsfLite {
  float qh0, ql0, qh1, ql1, G0, G1, G2, l2amp, sgn, rr, total;
  int lo0, hi0, lo1, hi1;
};

__device__ __forceinline__ PsfLite shfl_psf(const PsfLite &v, int src) {
  PsfLite o;
  const unsigned m = 0xffffffffu;
  o.qh0 = __shfl_sync(m, v.qh0, src);
  o.ql0 = __shfl_sync(m, v.ql0, src);
  o.qh1 = __shfl_sync(m, v.qh1, src);
  o.ql1 = __shfl_sync(m, v.ql1, src);
  o.G0 = __shfl_sync(m, v.G0, src);
  o.G1 = __shfl_sync(m, v.G1, src);
  o.G2 = __shfl_sync(m, v.G2, src);
  o.l2amp = __shfl_sync(m, v.l2amp, src);
  o.sgn = __shfl_sync(m, v.sgn, src);
  o.rr = __shfl_sync(m, v.rr, src);
  o.total = __shfl_sync(m, v.total, src);
  o.lo0 = __shfl_sync(m, v.lo0, src);
  o.hi0 = __shfl_sync(m, v.hi0, src);
  o.lo1 = __shfl_sync(m, v.lo1, src);
  o.hi1 = __shfl_sync(m, v.hi1, src);
  return o;
}

// Warp per (angle, tile), atoms in index order from the bitmap, lanes spread
// over each atom's cell box clipped to the tile, each cell's value by the
// quadrature rule; compensated shared-memory cell sums (deterministic).
template <int K>
__global__ void __launch_bounds__(kProjWarps * 32)
    gr_psf_project_kernel(Atoms at, Geom g, TileCfg tc, const uint32_t *bitmap, int W,
                          float s, ProjOut out) {
  extern __shared__ float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * kProjWarps + warp;
  if (item >= g.n_angles * tc.ntiles) return;
  const int cells = tc.t0 * tc.t1;
  float *acc = smem + (size_t)warp * kProjWarpFloats;
  float *cmp = acc + kTileCells;
  float *pc0 = cmp + kTileCells;
  float *pc1 = pc0 + 64;
  int *list = reinterpret_cast<int *>(pc1 + kTileDim1);
  const int a = item / tc.ntiles, t = item - a * tc.ntiles;
  const int tr = t / tc.nt1, tcix = t - tr * tc.nt1;
  const int r0 = tr * tc.t0, c0 = tcix * tc.t1;
  const int D0 = g.ax[0].n, D1 = (K == 1) ? 1 : g.ax[1].n;
  for (int e = lane; e < cells; e += 32) {
    acc[e] = 0.f;
    cmp[e] = 0.f;
  }
  for (int e = lane; e < tc.t0; e += 32)
    pc0[e] = (r0 + e < D0) ? g.ax[0].coords[r0 + e] : 0.f;
  if constexpr (K == 2)
    for (int e = lane; e < tc.t1; e += 32)
      pc1[e] = (c0 + e < D1) ? g.ax[1].coords[c0 + e] : 0.f;
  Frame<K> f;
  load_frame<K>(g.frames, a, f);
  __syncwarp();
  const uint32_t *words = bitmap + (size_t)item * W;
  for (int wb = 0; wb < W; wb += kListWords) {
    const int wi = wb + (lane < kListWords ? lane : 0);
    uint32_t wd = (lane < kListWords && wi < W) ? words[wi] : 0u;
    int cnt = __popc(wd), incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int pos = incl - cnt;
    while (wd) {
      const int b = __ffs(wd) - 1;
      list[pos++] = (wi << 5) + b;
      wd &= wd - 1;
    }
    __syncwarp();
    for (int bs = 0; bs < total; bs += 32) {
      const int idx = bs + lane;
      PsfLite mine{};
      mine.lo0 = 1;
      mine.hi0 = 0;
      mine.lo1 = 1;
      mine.hi1 = 0;
      if (idx < total) {
        const int j = list[idx];
        Pair<K> p;
        const bool ok = pair_setup<K>(at, j, f, g, p);
        PsfPair<K> q;
        psf_setup<K>(at, j, g, p, ok, s, q);
        mine.qh0 = p.qh[0];
        mine.ql0 = p.ql[0];
        mine.G0 = p.G[0];
        mine.G1 = p.G[1];
        mine.G2 = p.G[2];
        mine.l2amp = p.l2amp;
        mine.sgn = p.sgn;
        mine.rr = q.rr;
        mine.total = q.total;
        mine.lo0 = max(q.lo[0], r0);
        mine.hi0 = min(q.hi[0], r0 + tc.t0 - 1);
        if constexpr (K == 2) {
          mine.qh1 = p.qh[1];
          mine.ql1 = p.ql[1];
          mine.lo1 = max(q.lo[1], c0);
          mine.hi1 = min(q.hi[1], c0 + tc.t1 - 1);
        } else {
          mine.lo1 = 0;
          mine.hi1 = 0;
        }
      }
      const int nb = min(32, total - bs);
      for (int s2 = 0; s2 < nb; ++s2) {
        const PsfLite qq = shfl_psf(mine, s2);
        if (qq.lo0 > qq.hi0 || qq.lo1 > qq.hi1) continue;
        Pair<K> p;
        p.qh[0] = qq.qh0;
        p.ql[0] = qq.ql0;
        p.G[0] = qq.G0;
        p.G[1] = qq.G1;
        p.G[2] = qq.G2;
        p.l2amp = qq.l2amp;
        if constexpr (K == 2) {
          p.qh[1] = qq.qh1;
          p.ql[1] = qq.ql1;
        }
        PsfPair<K> q;
        q.rr = qq.rr;
        q.total = qq.total;
        const int bw = qq.hi1 - qq.lo1 + 1;
        const int ncell = (qq.hi0 - qq.lo0 + 1) * bw;
        const float inv_bw = 1.f / (float)bw;
        for (int e = lane; e < ncell; e += 32) {
          const int rr_ = (int)(((float)e + 0.5f) * inv_bw);
          const int cc = e - rr_ * bw;
          const int lr = qq.lo0 - r0 + rr_;
          const int lc = (K == 2) ? (qq.lo1 - c0 + cc) : 0;
          float dc[K], base[K], step[K];
          dc[0] = (pc0[lr] - qq.qh0) - qq.ql0;
          if constexpr (K == 2) dc[1] = (pc1[lc] - qq.qh1) - qq.ql1;
          const int kind = psf_cell_kind<K>(q, dc, s, base, step);
          if (kind == 0) continue;
          const float v = kind == 1 ? qq.total : qq.sgn * psf_quadrature<K>(p, base, step);
          const int ci = lr * tc.t1 + lc;
          const float s0 = acc[ci];
          const float tt = s0 + v;
          cmp[ci] += (fabsf(s0) >= fabsf(v)) ? ((s0 - tt) + v) : ((v - tt) + s0);
          acc[ci] = tt;
        }
        __syncwarp();
      }
    }
  }
  __syncwarp();
  float lsum = 0.f, lcmp = 0.f;
  for (int e = lane; e < cells; e += 32) {
    const int lr = e / tc.t1, lc = e - lr * tc.t1;
    const int row = r0 + lr, col = c0 + lc;
    if (row >= D0 || col >= D1) continue;
    const float v = acc[e] + cmp[e];
    const size_t gi = ((size_t)a * D0 + row) * D1 + col;
    if (out.R) out.R[gi] = v;
    float l = 0.f;
    if (out.epilogue == kEpiL2) {
      const float res = v - out.data[gi];
      if (out.alpha) out.alpha[gi] = res;
      l = 0.5f * res * res;
    } else if (out.epilogue == kEpiKL) {
      const float fo = out.data[gi];
      const float gg = v + out.bg;
      const float ig = 1.f / gg;
      if (out.alpha) out.alpha[gi] = 1.f - fo * ig;
      if (out.beta) out.beta[gi] = fo * ig * ig;
      l = kl_term(fo, gg);
    }
    const float tt = lsum + l;
    lcmp += (fabsf(lsum) >= fabsf(l)) ? ((lsum - tt) + l) : ((l - tt) + lsum);
    lsum = tt;
  }
  if (out.loss_part) {
    double d = warp_sum_d((double)lsum + (double)lcmp);
    if (lane == 0) out.loss_part[item] = d;
  }
}

// Fixed-order FP64 sum of n loss partials over many blocks (one block's FP64
// pipe, at 16 cycles per warp instruction, would take ~0.3 ms for the 640k
// partials of 20000 images): block b sums the contiguous segment
// [b seg, (b + 1) seg), each thread a strided part of it, then a fixed tree;
// the last block to finish reduces the block sums with a fixed tree.
// bsum: gridDim.x doubles (<= kLossMaxBlocks); done: a counter zeroed before
// the launch.
constexpr int kLossThreads = 256;
constexpr int kLossMaxBlocks = 256;
__global__ void __launch_bounds__(kLossThreads)
    gr_loss_finalize_kernel(const double *part, int n, double *out, double *bsum, int *done) {
  __shared__ double sh[kLossThreads];
  __shared__ int s_last;
  const int seg = (n + (int)gridDim.x - 1) / (int)gridDim.x;
  const int lo = blockIdx.x * seg, hi = min(n, lo + seg);
  double s = 0.0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    bsum[blockIdx.x] = sh[0];
    __threadfence();
    s_last = atomicAdd(done, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  sh[threadIdx.x] = (int)threadIdx.x < (int)gridDim.x ? __ldcg(bsum + threadIdx.x) : 0.0;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

// Tiling of the point-sampled 3D projection (Tuning::proj_form, key 3):
// 1: 16-row tiles (more resident warps), 2: 32-row tiles (fewer atoms cut
// by tile edges).
static int proj_rows(int form) { return form == 2 ? kTileDim0 : 16; }

// Loss partials of up to this many items are summed by the projection's
// last warp or block (sum_partials_warp: a chain of n / 256 FP64 adds);
// above it the 1024-thread gr_loss_finalize_kernel does it.
constexpr size_t kFusedLossItems = 8192;

// 3D problems of fewer detector cells (all angles) than
// Tuning::proj_split_cells (key 4; 0: never) split every tile's atoms over a
// block's warps.

template <int ROWS, int S, int NW>
static void launch_project3d(size_t items, const Atoms &at, const Geom &g, const TileCfg &tc,
                             const uint32_t *bitmap, int W, const ProjOut &o, int *next_item,
                             double *loss_out, const int *item_list, cudaStream_t stream) {
  constexpr size_t smem = kProjWarps * Proj3Smem<ROWS, S>::kFloats * sizeof(float);
  // with the few static bytes, below the 48 KB that needs no opt-in, so no
  // function attribute is set (safe under stream capture)
  static_assert(smem + 64 <= 48 * 1024, "smem");
  // persistent grid: the resident blocks of every SM, at most the blocks
  // that have an item to take
  static int resident[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (resident[dev] == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gr_project3d_kernel<ROWS, S, NW, false>,
                                                  kProjWarps * 32, smem);
    resident[dev] = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  }
  const size_t want = NW == 1 ? (items + kProjWarps - 1) / kProjWarps : items;
  const int grid = (int)(want < (size_t)resident[dev] ? want : (size_t)resident[dev]);
  if (item_list)
    gr_project3d_kernel<ROWS, S, NW, true><<<grid, kProjWarps * 32, smem, stream>>>(
        at, g, tc, bitmap, W, o, next_item, loss_out, item_list, next_item + 2);
  else
    gr_project3d_kernel<ROWS, S, NW, false><<<grid, kProjWarps * 32, smem, stream>>>(
        at, g, tc, bitmap, W, o, next_item, loss_out, nullptr, nullptr);
}

// rows: the tile's rows (3D) or cells (2D)
TileCfg make_tiles(int K, int D0, int D1, int rows) {
  TileCfg tc;
  if (K == 1) {
    tc.t0 = rows;
    tc.t1 = 1;
    tc.nt0 = (D0 + tc.t0 - 1) / tc.t0;
    tc.nt1 = 1;
  } else {
    tc.t0 = rows;
    tc.t1 = kTileDim1;
    tc.nt0 = (D0 + tc.t0 - 1) / tc.t0;
    tc.nt1 = (D1 + tc.t1 - 1) / tc.t1;
  }
  tc.ntiles = tc.nt0 * tc.nt1;
  return tc;
}

size_t project_skip_items(const Geom &g, int psf, const Tuning &t) {
  if (g.K != 2 || psf) return 0;
  const TileCfg tc = make_tiles(2, g.ax[0].n, g.ax[1].n, proj_rows(t.proj_form));
  return (size_t)g.n_angles * tc.ntiles;
}

size_t project_workspace_bytes(int K, int n_atoms, int n_angles, int D0, int D1,
                               const Tuning &t) {
  // sized for the smaller of the point-sampled and pixel-integrated tilings
  const int rows = K == 1 ? kTile1D
                          : (proj_rows(t.proj_form) < kTileDim0 ? proj_rows(t.proj_form)
                                                                : kTileDim0);
  TileCfg tc = make_tiles(K, D0, D1, rows);
  const size_t W = (size_t)(n_atoms + 31) / 32;
  const size_t items = (size_t)n_angles * tc.ntiles;
  // item counter of the persistent 3D kernel, finished-block counter, count
  // of listed items
  size_t bytes = align_up(4 * sizeof(int));
  // 3D: the bitmap is followed by a flag per item (cleared with it) and the
  // list of items some atom meets (a forward that skips the others)
  bytes += align_up(items * W * sizeof(uint32_t) + (K == 2 ? items * sizeof(uint32_t) : 0));
  bytes += align_up(items * sizeof(double));
  bytes += align_up(kLossMaxBlocks * sizeof(double));  // block sums of the loss finalize
  if (K == 1)  // per-(angle, atom) pair records of the 2D projection
    bytes += align_up((size_t)n_angles * (size_t)n_atoms * 2 * sizeof(float4));
  else
    bytes += align_up(items * sizeof(int));
  return bytes;
}

int launch_project(const Atoms &at, const Geom &g, const ProjOut &o_in,
                   double *loss_out, void *ws, size_t ws_bytes,
                   cudaStream_t stream, const Tuning &t) {
  const int K = g.K;
  const int D0 = g.ax[0].n, D1 = K == 1 ? 1 : g.ax[1].n;
  const int form = t.proj_form;
  // 2D: 64-cell tiles (two cells per lane) for form 2, 128 (four) for form
  // 3, else 32
  const bool wide2d = K == 1 && !o_in.psf && form == 2;
  const bool wide4 = K == 1 && !o_in.psf && form == 3;
  TileCfg tc = make_tiles(K, D0, D1,
                          K == 1 ? (wide4 ? 4 * kTile1D : wide2d ? 2 * kTile1D : kTile1D)
                                 : (!o_in.psf ? proj_rows(form) : kTileDim0));
  const int W = (at.n + 31) / 32;
  const size_t items = (size_t)g.n_angles * tc.ntiles;
  const size_t need = project_workspace_bytes(K, at.n, g.n_angles, D0, D1, t);
  // items no atom meets: point-sampled 3D only, fields only
  const int emode = o_in.empty_mode;
  if (emode != kEmptyNone &&
      (K != 2 || o_in.psf || o_in.R || !o_in.empty_loss || emode < 0 || emode > kEmptySkip))
    return kErrArg;
  const bool record = emode == kEmptyRecord;
  if (ws_bytes < need || (ws == nullptr && need > 0)) return kErrWorkspace;
  char *wp = static_cast<char *>(ws);
  int *next_item = reinterpret_cast<int *>(wp);
  wp += align_up(4 * sizeof(int));
  uint32_t *bitmap = reinterpret_cast<uint32_t *>(wp);
  uint32_t *flag = bitmap + items * W;  // 3D: one per item
  wp += align_up(items * W * sizeof(uint32_t) + (K == 2 ? items * sizeof(uint32_t) : 0));
  double *loss_part = reinterpret_cast<double *>(wp);
  wp += align_up(items * sizeof(double)) + align_up(kLossMaxBlocks * sizeof(double));
  float4 *pairs = K == 1 ? reinterpret_cast<float4 *>(wp) : nullptr;
  int *item_list = K == 2 ? reinterpret_cast<int *>(wp) : nullptr;
  const bool skip = emode == kEmptySkip;
  // one clear covers the counters and the bitmap (and the item flags)
  if (cudaMemsetAsync(ws, 0,
                      align_up(4 * sizeof(int)) + items * W * sizeof(uint32_t) +
                          (skip ? items * sizeof(uint32_t) : 0),
                      stream) != cudaSuccess)
    return kErrLaunch;
  ProjOut o = o_in;
  o.loss_part = loss_out ? loss_part : nullptr;
  // skipping: the items no atom meets take their recorded loss partials
  // (copied first, the listed items' partials overwrite theirs)
  if (skip && o.loss_part &&
      cudaMemcpyAsync(o.loss_part, o_in.empty_loss, items * sizeof(double),
                      cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
    return kErrLaunch;
  if (record) {
    // every item as if no atom met it: its loss partial goes to empty_loss,
    // under the schedule (split, tiling) of a forward of these atoms, so it
    // equals bitwise what that forward computes for an empty item
    o.alpha = o.beta = nullptr;
    o.loss_part = o_in.empty_loss;
    loss_out = nullptr;
  }
  // half-width of the (square) cells of the pixel-integrated operator
  const float psf_s = 0.5f / g.ax[0].inv_step;
  if (W > 0 && !record) {
    dim3 bgrid((at.n + 127) / 128, g.n_angles);
    if (o.psf) {
      if (K == 1) gr_psf_bin_kernel<1><<<bgrid, 128, 0, stream>>>(at, g, tc, bitmap, W, psf_s);
      else gr_psf_bin_kernel<2><<<bgrid, 128, 0, stream>>>(at, g, tc, bitmap, W, psf_s);
    } else if (K == 1) {
      gr_bin_kernel<1><<<bgrid, 128, 0, stream>>>(at, g, tc, bitmap, W, pairs, nullptr, nullptr,
                                                  nullptr);
    } else {
      gr_bin_kernel<2><<<bgrid, 128, 0, stream>>>(at, g, tc, bitmap, W, nullptr,
                                                  skip ? flag : nullptr, item_list,
                                                  next_item + 2);
    }
    note_launches(1);
  }
  const int blocks = (int)((items + kProjWarps - 1) / kProjWarps);
  const size_t smem = (size_t)kProjWarps * kProjWarpFloats * sizeof(float);
  // smem (kProjWarps * kProjWarpFloats floats) stays below the 48 KB that
  // needs no opt-in, so no function attribute is set (safe under capture)
  static_assert(kProjWarps * kProjWarpFloats * sizeof(float) <= 48 * 1024, "smem");
  bool fused_loss = false;
  timer_mark(1, 0, stream);
  if (o.psf) {
    if (K == 1)
      gr_psf_project_kernel<1><<<blocks, kProjWarps * 32, smem, stream>>>(at, g, tc, bitmap, W, psf_s, o);
    else
      gr_psf_project_kernel<2><<<blocks, kProjWarps * 32, smem, stream>>>(at, g, tc, bitmap, W, psf_s, o);
  } else if (K == 1) {
    // one block per (angle, tile) item; for up to kFusedLossItems tiles the
    // last block also sums the loss partials (no separate finalize launch)
    fused_loss = loss_out != nullptr && items <= kFusedLossItems;
    double *lo = fused_loss ? loss_out : nullptr;
    if (wide4 && W >= 8)
      gr_project1d_kernel<true, 8, 4, 2><<<(unsigned)items, 8 * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
    else if (wide4)
      gr_project1d_kernel<true, kProjWarps, 4><<<(unsigned)items, kProjWarps * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
    else if (wide2d && W >= 8)
      gr_project1d_kernel<true, 8, 2, 2><<<(unsigned)items, 8 * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
    else if (wide2d)
      gr_project1d_kernel<true, kProjWarps, 2><<<(unsigned)items, kProjWarps * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
    else if (W >= 32)  // 1024 atoms up: four list entries per thread
      gr_project1d_kernel<true, 8, 1, 4><<<(unsigned)items, 8 * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
    else if (W >= 8)  // 8 warps share a tile's atoms from 8 bitmap words (256 atoms) up
      gr_project1d_kernel<true, 8, 1, 2><<<(unsigned)items, 8 * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
    else
      gr_project1d_kernel<true, kProjWarps><<<(unsigned)items, kProjWarps * 32, 0, stream>>>(
          at, g, tc, bitmap, W, o, lo, next_item + 1, pairs);
  } else {
    // the split is chosen from the problem's size alone (not from the
    // tiling), so both tilings keep giving the same cell sums
    const bool split = t.proj_split_cells > 0 && W >= kProjWarps &&
                       (size_t)g.n_angles * D0 * D1 < (size_t)t.proj_split_cells;
    fused_loss = loss_out != nullptr && items <= kFusedLossItems;
    double *lo = fused_loss ? loss_out : nullptr;
    const int Wk = record ? 0 : W;  // recording: no atom in any item
    // skipping: only the listed items (none without atoms)
    const int *il = skip ? item_list : nullptr;
    if (form == 2) {
      if (split) launch_project3d<32, 34, kProjWarps>(items, at, g, tc, bitmap, Wk, o, next_item, lo, il, stream);
      else launch_project3d<32, 34, 1>(items, at, g, tc, bitmap, Wk, o, next_item, lo, il, stream);
    } else {
      if (split) launch_project3d<16, 37, kProjWarps>(items, at, g, tc, bitmap, Wk, o, next_item, lo, il, stream);
      else launch_project3d<16, 37, 1>(items, at, g, tc, bitmap, Wk, o, next_item, lo, il, stream);
    }
  }
  timer_mark(1, 1, stream);
  note_launches(1);
  if (loss_out && !fused_loss) {
    // about 8 partials per thread, at most kLossMaxBlocks blocks; the
    // finished-block counter (next_item + 1) is unused when the loss is not
    // fused into the projection
    size_t lb = (items + kLossThreads * 8 - 1) / (kLossThreads * 8);
    lb = lb < 1 ? 1 : (lb > kLossMaxBlocks ? kLossMaxBlocks : lb);
    double *bsum = loss_part + align_up(items * sizeof(double)) / sizeof(double);
    gr_loss_finalize_kernel<<<(unsigned)lb, kLossThreads, 0, stream>>>(loss_part, (int)items,
                                                                        loss_out, bsum,
                                                                        next_item + 1);
    note_launches(1);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

// ---- multi-problem launches (2D) -------------------------------------------
// Blocks of problems whose fit has stopped return at once (the whole block).
__global__ void __launch_bounds__(128)
    gr_batch_bin_kernel(const BatchProb *__restrict__ probs, const int *__restrict__ off, int n,
                        const int *__restrict__ active, int use_trial) {
  const int p = batch_find(off, n, blockIdx.x);
  if (!active[p]) return;
  const BatchProb &B = probs[p];
  const int lb = blockIdx.x - off[p];
  const int bxn = (B.cur.n + 127) / 128;
  bin_body<1>(use_trial ? B.trial : B.cur, B.g, B.tc, B.bitmap, B.W, B.pairs, lb % bxn,
              lb / bxn);
}

__global__ void __launch_bounds__(kProjWarps * 32)
    gr_batch_project_kernel(const BatchProb *__restrict__ probs, const int *__restrict__ off,
                            int n, const int *__restrict__ active, int use_trial) {
  const int p = batch_find(off, n, blockIdx.x);
  if (!active[p]) return;
  const BatchProb &B = probs[p];
  project1d_body<true, kProjWarps>(use_trial ? B.trial : B.cur, B.g, B.tc, B.bitmap, B.W, B.out,
                                   use_trial ? B.loss_trial : B.loss_cur, B.done, B.pairs,
                                   blockIdx.x - off[p], B.items);
}

int launch_batch_bin(const BatchLaunch &b, int use_trial, cudaStream_t stream) {
  if (b.grid_bin <= 0) return kOk;
  gr_batch_bin_kernel<<<b.grid_bin, 128, 0, stream>>>(b.probs, b.off_bin, b.n, b.active,
                                                      use_trial);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int launch_batch_project(const BatchLaunch &b, int use_trial, cudaStream_t stream) {
  if (b.grid_proj <= 0) return kOk;
  gr_batch_project_kernel<<<b.grid_proj, kProjWarps * 32, 0, stream>>>(
      b.probs, b.off_proj, b.n, b.active, use_trial);
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int preload_project() {
  return preload_fn(gr_bin_kernel<1>) + preload_fn(gr_bin_kernel<2>) +
         preload_fn(gr_psf_bin_kernel<1>) + preload_fn(gr_psf_bin_kernel<2>) +
         preload_fn(gr_project3d_kernel<16, 37, 1, false>) +
         preload_fn(gr_project3d_kernel<16, 37, kProjWarps, false>) +
         preload_fn(gr_project3d_kernel<32, 34, 1, false>) +
         preload_fn(gr_project3d_kernel<32, 34, kProjWarps, false>) +
         preload_fn(gr_project3d_kernel<16, 37, 1, true>) +
         preload_fn(gr_project3d_kernel<16, 37, kProjWarps, true>) +
         preload_fn(gr_project3d_kernel<32, 34, 1, true>) +
         preload_fn(gr_project3d_kernel<32, 34, kProjWarps, true>) +
         preload_fn(gr_project1d_kernel<true, 8, 1, 4>) +
         preload_fn(gr_project1d_kernel<true, 8, 1, 2>) +
         preload_fn(gr_project1d_kernel<true, kProjWarps>) +
         preload_fn(gr_project1d_kernel<true, 8, 2, 2>) +
         preload_fn(gr_project1d_kernel<true, kProjWarps, 2>) +
         preload_fn(gr_project1d_kernel<true, 8, 4, 2>) +
         preload_fn(gr_project1d_kernel<true, kProjWarps, 4>) +
         preload_fn(gr_psf_project_kernel<1>) + preload_fn(gr_psf_project_kernel<2>) +
         preload_fn(gr_loss_finalize_kernel) + preload_fn(gr_batch_bin_kernel) +
         preload_fn(gr_batch_project_kernel);
}

}  // namespace gr
