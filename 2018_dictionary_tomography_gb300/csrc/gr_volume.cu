// Rendering atoms on a voxel grid (sm_103a).
//
// Replaces __VolProj (GaussDictCode/bin/NewtonBases2D.py:261-271,
// GaussDictCode/bin/NewtonBases.py:700-711), which evaluates every atom at
// every voxel:  u(y) = sum_j I_j sqrt(30/pi) exp(-30 |r_j (y - x_j)|^2) where
// |r_j (y - x_j)| <= 1, else 0 (NewtonBases.py:42-46).
// One CTA per voxel tile; the CTA scans the atoms in index order, keeps those
// whose support box (the ellipsoid |r (y - x)| <= 1, whose half-extent along
// axis i is the norm of row i of r^{-1}) meets the tile, compacting them into
// shared memory in atom order; each thread owns one voxel and adds the listed
// atoms in that order.  Deterministic, no atomics.  Coordinate vectors must be
// monotone (the tile box is read from the tile's end coordinates).
#include "gr_kernels.cuh"

namespace gr {

constexpr int kVolThreads = 256;

struct VolGrid {
  int n[3];
  const float *y[3];
};

// Voxel-integrated value of one atom (point_spread_functions.py __if2 :425,
// __if3 :459): 11^D-point rule over the voxel of half-width s clipped to the
// box +-rr (rr = 1 / min diag r) around the atom, points at lo + t (hi-lo)/10
// (t = 1..11), no cut-off; total mass inside, zero beyond rr + s.
template <int D>
__device__ __forceinline__ float psf_voxel(float Iv, const float *X, const float (&M)[3][3],
                                           float rr, float total, float s) {
  float n2 = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) n2 = fmaf(X[i], X[i], n2);
  const float n = sqrtf(n2);
  if (n + rr < s) return total;
  if (n - rr > s) return 0.f;
  float lo[3], st[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float l = fmaxf(X[i] - rr, -s), h = fminf(X[i] + rr, s);
    st[i] = 0.1f * (h - l);
    lo[i] = l;
  }
  float sum = 0.f;
  for (int a = 1; a <= 11; ++a) {
    const float Y0 = fmaf((float)a, st[0], lo[0]) - X[0];
    for (int b = 1; b <= 11; ++b) {
      const float Y1 = fmaf((float)b, st[1], lo[1]) - X[1];
      if (D == 2) {
        const float p0 = M[0][0] * Y0 + M[0][1] * Y1, p1 = M[1][1] * Y1;
        sum += ex2_approx((p0 * p0 + p1 * p1) * kNegThirtyLog2e);
      } else {
#pragma unroll
        for (int c = 1; c <= 11; ++c) {
          const float Y2 = fmaf((float)c, st[2], lo[2]) - X[2];
          const float p0 = M[0][0] * Y0 + M[0][1] * Y1 + M[0][2] * Y2;
          const float p1 = M[1][1] * Y1 + M[1][2] * Y2, p2 = M[2][2] * Y2;
          sum += ex2_approx((p0 * p0 + p1 * p1 + p2 * p2) * kNegThirtyLog2e);
        }
      }
    }
  }
  constexpr float kNorm = 3.0901936161855166f;  // sqrt(30 / pi)
  return D == 2 ? Iv * kNorm * sum * (100.f * st[0] * st[1] / 121.f)
                : Iv * kNorm * sum * (1000.f * st[0] * st[1] * st[2] / 1331.f);
}

template <int D, bool PSF>
__global__ void __launch_bounds__(kVolThreads)
    gr_volproj_kernel(Atoms at, VolGrid vg, int t0, int t1, int t2, float s, float *u) {
  __shared__ float sI[kVolThreads], sx[3][kVolThreads], sr[6][kVolThreads];
  __shared__ int wcount[kVolThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // tile extents: D == 3: t0 x t1 x t2 voxels; D == 2: t0 x t1
  const int nt1 = (vg.n[1] + t1 - 1) / t1;
  const int nt2 = D == 3 ? (vg.n[2] + t2 - 1) / t2 : 1;
  int b = blockIdx.x;
  const int b2 = b % nt2;
  b /= nt2;
  const int b1 = b % nt1, b0 = b / nt1;
  const int o0 = b0 * t0, o1 = b1 * t1, o2 = b2 * (D == 3 ? t2 : 1);
  // this thread's voxel
  const int l2 = D == 3 ? tid % t2 : 0;
  const int l1 = D == 3 ? (tid / t2) % t1 : tid % t1;
  const int l0 = D == 3 ? tid / (t1 * t2) : tid / t1;
  const int i0 = o0 + l0, i1 = o1 + l1, i2 = o2 + l2;
  const bool inside = i0 < vg.n[0] && i1 < vg.n[1] && (D == 2 || i2 < vg.n[2]);
  float yv[3] = {0.f, 0.f, 0.f};
  if (inside) {
    yv[0] = vg.y[0][i0];
    yv[1] = vg.y[1][i1];
    if (D == 3) yv[2] = vg.y[2][i2];
  }
  // coordinate box of the tile
  float blo[3], bhi[3];
  {
    const int e0 = min(o0 + t0, vg.n[0]) - 1, e1 = min(o1 + t1, vg.n[1]) - 1;
    const float a0 = vg.y[0][o0], c0 = vg.y[0][e0], a1 = vg.y[1][o1], c1 = vg.y[1][e1];
    blo[0] = fminf(a0, c0); bhi[0] = fmaxf(a0, c0);
    blo[1] = fminf(a1, c1); bhi[1] = fmaxf(a1, c1);
    if (D == 3) {
      const int e2 = min(o2 + t2, vg.n[2]) - 1;
      const float a2 = vg.y[2][o2], c2 = vg.y[2][e2];
      blo[2] = fminf(a2, c2); bhi[2] = fmaxf(a2, c2);
    }
  }
  constexpr float kNorm = 3.0901936161855166f;  // sqrt(30 / pi)
  float acc = 0.f;
  for (int base = 0; base < at.n; base += kVolThreads) {
    const int j = base + tid;
    bool hit = false;
    float M[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float xj[3] = {0.f, 0.f, 0.f};
    if (j < at.n) {
      float Mk[D][D];
      load_r<D - 1>(at, j, Mk);
#pragma unroll
      for (int a = 0; a < D; ++a)
#pragma unroll
        for (int c = 0; c < D; ++c) M[a][c] = Mk[a][c];
#pragma unroll
      for (int i = 0; i < D; ++i) xj[i] = at.x[(size_t)D * j + i];
      // rows of r^{-1} for the upper-triangular r (back substitution)
      float inv[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      bool ok = true;
#pragma unroll
      for (int i = 0; i < D; ++i) ok = ok && M[i][i] != 0.f;
      if (ok) {
#pragma unroll
        for (int c = D - 1; c >= 0; --c) {
          inv[c][c] = 1.f / M[c][c];
#pragma unroll
          for (int rr = c - 1; rr >= 0; --rr) {
            float s = 0.f;
#pragma unroll
            for (int k = rr + 1; k <= c; ++k) s += M[rr][k] * inv[k][c];
            inv[rr][c] = -s / M[rr][rr];
          }
        }
        hit = true;
        float rr = M[0][0];
#pragma unroll
        for (int i = 1; i < D; ++i) rr = fminf(rr, M[i][i]);
        rr = 1.f / rr;
#pragma unroll
        for (int i = 0; i < D; ++i) {
          float e = 0.f;
#pragma unroll
          for (int k = 0; k < D; ++k) e += inv[i][k] * inv[i][k];
          e = PSF ? (rr + s) * 1.0001f : sqrtf(e) * 1.0001f;
          hit = hit && (xj[i] + e >= blo[i]) && (xj[i] - e <= bhi[i]);
        }
      }
    }
    // ordered compaction of the hits of this chunk
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) wcount[warp] = __popc(bal);
    __syncthreads();
    int off = 0, total = 0;
    for (int w = 0; w < kVolThreads / 32; ++w) {
      if (w < warp) off += wcount[w];
      total += wcount[w];
    }
    if (hit) {
      const int pos = off + __popc(bal & ((1u << lane) - 1u));
      sI[pos] = at.I[j] * kNorm;
#pragma unroll
      for (int i = 0; i < 3; ++i) sx[i][pos] = xj[i];
      sr[0][pos] = M[0][0];
      sr[1][pos] = M[1][1];
      sr[2][pos] = M[0][1];
      if (D == 3) {
        sr[2][pos] = M[2][2];
        sr[3][pos] = M[0][1];
        sr[4][pos] = M[1][2];
        sr[5][pos] = M[0][2];
      }
    }
    __syncthreads();
    if (inside) {
      for (int k = 0; k < total; ++k) {
        const float Y0 = yv[0] - sx[0][k], Y1 = yv[1] - sx[1][k];
        float nn;
        if (D == 2) {
          const float a = sr[0][k] * Y0 + sr[2][k] * Y1, c = sr[1][k] * Y1;
          nn = a * a + c * c;
        } else {
          const float Y2 = yv[2] - sx[2][k];
          const float a = sr[0][k] * Y0 + sr[3][k] * Y1 + sr[5][k] * Y2;
          const float c = sr[1][k] * Y1 + sr[4][k] * Y2;
          const float d = sr[2][k] * Y2;
          nn = a * a + c * c + d * d;
        }
        if (!PSF && nn <= 1.f) acc += sI[k] * ex2_approx(nn * kNegThirtyLog2e);
        if (PSF) {
          float Mk[3][3] = {{sr[0][k], D == 2 ? sr[2][k] : sr[3][k], D == 2 ? 0.f : sr[5][k]},
                            {0.f, sr[1][k], D == 2 ? 0.f : sr[4][k]},
                            {0.f, 0.f, D == 2 ? 0.f : sr[2][k]}};
          float X[3] = {sx[0][k] - yv[0], sx[1][k] - yv[1], D == 3 ? sx[2][k] - yv[2] : 0.f};
          float mn = Mk[0][0];
#pragma unroll
          for (int i = 1; i < D; ++i) mn = fminf(mn, Mk[i][i]);
          const float rr = 1.f / mn;
          constexpr float kNormV = 3.0901936161855166f;
          const float Iv = sI[k] / kNormV;
          const float det = D == 2 ? Mk[0][0] * Mk[1][1] : Mk[0][0] * Mk[1][1] * Mk[2][2];
          const float total = D == 2 ? Iv / det * 0.32360019f : Iv / det * 0.10471976f;
          acc += psf_voxel<D>(Iv, X, Mk, rr, total, s);
        }
      }
    }
    __syncthreads();
  }
  if (inside) {
    const size_t gi = D == 3 ? (((size_t)i0 * vg.n[1] + i1) * vg.n[2] + i2)
                             : ((size_t)i0 * vg.n[1] + i1);
    u[gi] = acc;
  }
}

int launch_volproj(const Atoms &at, int dim, const int *n, const float *const *y,
                   float *u, int psf, float s, cudaStream_t stream) {
  VolGrid vg;
  for (int k = 0; k < 3; ++k) {
    vg.n[k] = k < dim ? n[k] : 1;
    vg.y[k] = k < dim ? y[k] : nullptr;
  }
  if (dim == 2) {
    const int t0 = 16, t1 = 16;
    const int blocks = ((vg.n[0] + t0 - 1) / t0) * ((vg.n[1] + t1 - 1) / t1);
    if (psf) gr_volproj_kernel<2, true><<<blocks, kVolThreads, 0, stream>>>(at, vg, t0, t1, 1, s, u);
    else gr_volproj_kernel<2, false><<<blocks, kVolThreads, 0, stream>>>(at, vg, t0, t1, 1, s, u);
  } else {
    const int t0 = 4, t1 = 8, t2 = 8;
    const int blocks = ((vg.n[0] + t0 - 1) / t0) * ((vg.n[1] + t1 - 1) / t1) *
                       ((vg.n[2] + t2 - 1) / t2);
    if (psf) gr_volproj_kernel<3, true><<<blocks, kVolThreads, 0, stream>>>(at, vg, t0, t1, t2, s, u);
    else gr_volproj_kernel<3, false><<<blocks, kVolThreads, 0, stream>>>(at, vg, t0, t1, t2, s, u);
  }
  note_launches(1);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrLaunch;
}

int preload_volume() {
  return preload_fn(gr_volproj_kernel<2, false>) + preload_fn(gr_volproj_kernel<3, false>) +
         preload_fn(gr_volproj_kernel<2, true>) + preload_fn(gr_volproj_kernel<3, true>);
}

}  // namespace gr
