// Declarations shared by the kernel translation units and the C ABI.
#pragma once
#include <atomic>

#include "gr_common.cuh"

namespace gr {

// ---- forward projection tiling -------------------------------------------
constexpr int kProjWarps = 4;        // independent (angle, tile) warps per CTA
constexpr int kTileDim0 = 32;        // 3D tile rows (detector axis 0)
constexpr int kTileDim1 = 32;        // 3D tile cols (detector axis 1, contiguous)
constexpr int kTile1D = 32;          // 2D tile length (one cell per lane)
constexpr int kTileCells = 1024;     // shared-memory cell sums per warp
constexpr int kListWords = 16;       // bitmap words compacted per pass
constexpr int kProjWarpFloats =
    2 * kTileCells + 64 + kTileDim1 + kListWords * 32;

// Parameters of a per-atom regulariser (gr_reg.cu).
struct RegParams {
  double p[8];
};

struct TileCfg {
  int t0, t1;     // tile extent along detector axes 0 and 1
  int nt0, nt1;   // tiles along each axis
  int ntiles;
};

enum Epilogue : int { kEpiNone = 0, kEpiL2 = 1, kEpiKL = 2 };

struct ProjOut {
  float *R;            // sinogram (nullable)
  int epilogue;
  const float *data;   // data sinogram (L2 / KL)
  float bg;            // KL background
  float *alpha;        // first-order weight field (nullable)
  float *beta;         // Gauss-Newton weight field (KL, nullable)
  double *loss_part;   // per-(angle, tile) loss partials (set by the launcher)
  int psf;             // 1: pixel-integrated values (point-spread operator)
  // Items no atom meets (point-sampled 3D only; R not written):
  // kEmptyRecord writes every item's loss with no atom in it to empty_loss
  // and no field; kEmptySkip gives an item whose bitmap is empty the loss
  // recorded in empty_loss and leaves its fields unwritten.
  int empty_mode;
  double *empty_loss;
};
enum EmptyMode : int { kEmptyNone = 0, kEmptyRecord = 1, kEmptySkip = 2 };

// ---- derivatives -----------------------------------------------------------
enum DerivMode : int {
  kModeField = 0,    // alpha / beta fields given (fit derivatives)
  kModeL2Atom = 1,   // alpha = R_atom - C, beta = 1 (per-atom L2 fit to C)
  kModeInner = 2,    // alpha = C, beta = 0 (inner product <R_atom, C>)
};

struct DerivIn {
  int mode;
  int order;             // 1: value + gradient, 2: + Hessian
  const float *alpha;    // field, or C for kModeL2Atom / kModeInner
  const float *beta;     // field (nullable)
  float beta_const;      // used when beta == nullptr
  int psf;               // 1: pixel-integrated operator
};

struct DerivOut {
  double *f;   // (N)
  double *g;   // (N, P_out)
  double *H;   // (N, P_out, P_out), order 2
};

// Work split of a derivative launch (gr_derivs.cu, deriv_cfg).
struct DerivCfg {
  int ag;       // distinct atoms per warp (power of two)
  int sg;       // lanes per atom (32 / ag)
  int ch;       // angles per chunk
  int nchunks;
  int qn;       // partial values per atom
  int rs;       // lanes sharing one (atom, angle) pair's cells (power of two)
};

inline size_t align_up(size_t b) { return (b + 255) & ~(size_t)255; }

// Work-split and tiling schedule of the projection and derivative launches
// (keys of gr_set_tuning / gr_plan_set).  g_tuning is the process-wide
// default; a gr_plan carries its own copy, so launches on different streams
// can run different schedules at once.
struct Tuning {
  int deriv_target_warps = 131072;  // key 0
  int deriv_min_angles = 1;         // key 1
  int deriv_atoms_per_warp = 0;     // key 2 (0: automatic)
  int proj_form = 1;                // key 3 (3D 1: 16 x 32 tiles, 2: 32 x 32; 2D 32, 64, 128 cells)
  int proj_split_cells = 4 << 20;   // key 4
  int deriv_split_lanes = 65536;    // key 6
  int deriv_one_mb = 1024;          // key 7
  int deriv_wide_rows = 0;          // key 8 (1: 3D Hessian rows in 8-cell chunks)
  int deriv_block_warps = 1;        // key 9 (warps per block, one-angle-per-lane kernels)
};
extern Tuning g_tuning;
int tuning_set(Tuning &t, int key, int value);
int tuning_get(const Tuning &t, int key);

TileCfg make_tiles(int K, int D0, int D1, int rows);
// (angle, tile) items of a forward that can skip items no atom meets (the
// point-sampled 3D projection under t's tiling; 0 for the others)
size_t project_skip_items(const Geom &g, int psf, const Tuning &t = g_tuning);
size_t project_workspace_bytes(int K, int n_atoms, int n_angles, int D0, int D1,
                               const Tuning &t = g_tuning);
int launch_project(const Atoms &at, const Geom &g, const ProjOut &o,
                   double *loss_out, void *ws, size_t ws_bytes,
                   cudaStream_t stream, const Tuning &t = g_tuning);

size_t derivs_workspace_bytes(int K, int n_atoms, int n_angles, int order,
                              const Tuning &t = g_tuning);
DerivCfg deriv_cfg(int K, int n_atoms, int n_angles, int order, const Tuning &t,
                   bool split = true);
int finalize_blocks(int n_atoms);   // grid of the derivative finalize launch
int launch_derivs(const Atoms &at, const Geom &g, const DerivIn &in,
                  const DerivOut &out, void *ws, size_t ws_bytes,
                  cudaStream_t stream, const Tuning &t = g_tuning);

int launch_sum_squares(const float *C, size_t n, double *out, void *ws,
                       size_t ws_bytes, cudaStream_t stream);

int launch_count(const Atoms &at, const Geom &g, unsigned long long *out,
                 cudaStream_t stream);
int launch_ex2_probe(int blocks, int threads, int iters, float *out,
                     cudaStream_t stream);

int launch_atom_update(const Atoms &olda, const Atoms &newa, const Geom &g, int fit,
                       int apply, float *R, const float *data, float bg, float *alpha,
                       float *beta, double *dloss, void *ws, size_t ws_bytes,
                       cudaStream_t stream);
struct AtomOut {
  float *I, *x, *r;
};
struct AtomIn {
  const float *I, *x, *r;
};
int launch_newton_solve(int dim, int iso, int n, const double *g, const double *H,
                        const double *lam, const double *theta,
                        const unsigned char *mask, double *theta_new,
                        double *step_norm, int *fail, AtomOut ao, cudaStream_t stream);
// fit fields adopted with an accepted trial (all null: none)
struct FieldCopy {
  const float *alpha_t;
  float *alpha;
  const float *beta_t;
  float *beta;
  size_t n;
};
int launch_newton_accept(int n, int P, int pr, int dim, double *loss_cur,
                         const double *loss_trial, double *theta,
                         const double *theta_trial, double *lam, double lam_min,
                         double lam_max, AtomOut cur, AtomIn trial, double *hist,
                         int *hist_acc, int *counter, int hist_len, FieldCopy fc,
                         cudaStream_t stream);

int launch_volproj(const Atoms &at, int dim, const int *n, const float *const *y,
                   float *u, int psf, float s, cudaStream_t stream);

// ---- multi-problem launches (gr_loop.cu builds them) -----------------------
// One 2D L2 damped-Newton problem of a multi-problem launch: its device
// buffers and launch shapes.  A table of them lives in device memory, and
// each kernel of the batched iteration maps its blocks to (problem, block of
// that problem) through per-kernel block offsets, then runs the same block
// body as the problem's own launch would: every problem gets the results it
// gets alone.
struct BatchProb {
  Atoms cur, trial;
  Geom g;
  TileCfg tc;
  int W, items;                 // bitmap words per tile, (angle, tile) items
  ProjOut out;                  // data, fit fields, loss partials (L2 epilogue)
  uint32_t *bitmap;
  float4 *pairs;
  int *done;                    // finished-block counter of the projection
  double *loss_cur, *loss_trial;
  DerivIn din;                  // field mode on the fit fields, order 2
  DerivCfg cfg;
  float *part;                  // derivative chunk partials
  DerivOut dout;                // f, g, H of the current atoms
  double *theta, *theta_trial, *lam, *step;
  double *hist;
  int *hist_acc, *counter;
  int hist_len, max_iter;
  double tol, lam_min, lam_max;
  int P, pr;                    // parameters and r entries per atom
};

// The device tables of a batch: per kernel, off[p] is problem p's first
// block and off[n] the launch's grid.
struct BatchLaunch {
  const BatchProb *probs;
  int n;
  int *active;                  // 1 while problem p's fit runs
  const int *off_bin, *off_proj, *off_deriv, *off_fin, *off_solve, *off_acc;
  int grid_bin, grid_proj, grid_deriv, grid_fin, grid_solve, grid_acc;
};

// the problem owning block b: the last p with off[p] <= b (off[0] = 0,
// b < off[n]; problems of no blocks are skipped)
__device__ __forceinline__ int batch_find(const int *off, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct Batch;
// workspace of a batch of these problems (0: a problem cannot be batched)
size_t batch_workspace_bytes(const BatchProb *probs, int n);
// probs: atoms, geometry and the caller's per-problem buffers filled in; the
// launch shapes and workspace pointers are set here
int batch_create(const BatchProb *probs, int n, void *ws, size_t ws_bytes, int max_reject,
                 cudaStream_t stream, Batch **out);
int launch_batch_bin(const BatchLaunch &b, int use_trial, cudaStream_t stream);
int launch_batch_project(const BatchLaunch &b, int use_trial, cudaStream_t stream);
int launch_batch_derivs(const BatchLaunch &b, cudaStream_t stream);
int launch_batch_solve(const BatchLaunch &b, int P, cudaStream_t stream);
int launch_batch_accept(const BatchLaunch &b, cudaStream_t stream);


// host-side count of kernels launched by this library
void note_launches(int n);

// Loads a kernel's code now.  Module loading is lazy by default, so a
// kernel's first launch -- or the first instantiation of a graph holding it
// -- would otherwise pay the load while other work waits.  Returns 1 on
// failure.
template <typename F>
inline int preload_fn(F f) {
  cudaFuncAttributes a;
  return cudaFuncGetAttributes(&a, f) == cudaSuccess ? 0 : 1;
}
// per-file preloads of every kernel a file launches (failure counts)
int preload_project();
int preload_derivs();
int preload_update();
int preload_loop();
int preload_moments();
int preload_reg();
int preload_volume();
int launch_accept_fields(const double *loss_cur, const double *loss_trial, const float *alpha_t,
                         float *alpha, const float *beta_t, float *beta, size_t n,
                         cudaStream_t stream);
int launch_moments(const Geom &g, const float *res, const float *rr, float t, float scale,
                   double *S0, double *S1, double *S2, cudaStream_t stream);
// kernel timers (which: 1 projection kernel, 2 derivative kernel)
void timer_mark(int which, int end, cudaStream_t stream);
int timer_enable(int which, int enable);
int timer_read(int which, double *total_ms, int *launches);
extern std::atomic<unsigned long long> g_launches;

}  // namespace gr
