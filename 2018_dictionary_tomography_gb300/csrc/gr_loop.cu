// Device-resident fitting loop (sm_103a): one CUDA graph per fitting problem
// whose WHILE conditional node repeats a captured damped-Newton iteration
// until a stop test on the device clears the condition.
//
// The reference drives its Newton loop from the host, one kernel launch per
// atom and a host decision per step (GaussDictCode/NewtonGaussian.py:18-109).
// Here the caller captures one iteration (projection + fit, per-atom
// derivatives, FP64 block solves, trial projection, device-side accept; all
// on one stream) into the body of a WHILE node; gr_fit_loop_end appends
// gr_fit_loop_stop_kernel, which reads the loss history that the accept
// kernel writes and decides on the device whether to run another iteration.
// A whole fit is then one graph launch with no host round trip.  Inside the
// iteration, gr_fit_loop_gate_begin / _end put the derivative evaluation into
// the body of an IF node that a gate kernel opens only after an accepted
// trial (or on the first iteration): a rejected trial leaves the atoms and
// so their derivatives unchanged.
//
// Termination does not depend on the fit: the stop kernel counts the body's
// executions in its own guard word (cleared by a memset node ahead of the
// WHILE node at every launch) and stops after guard_max of them whatever the
// history says.
#include <cuda_runtime.h>

#include <new>
#include <vector>

#include "gr_kernels.cuh"

namespace gr {

struct FitLoop {
  cudaGraph_t graph = nullptr;
  cudaGraph_t body = nullptr;  // owned by graph
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle handle = 0;
  int *guard = nullptr;
  bool capturing = false;
  bool captured_ok = false;
  // an IF node in the body whose work runs only when the atoms moved
  cudaGraphConditionalHandle gate = 0;
  cudaGraphNode_t gate_node = nullptr;
  bool gated = false;          // capturing into the IF node's body now
  bool failed = false;         // a gate step failed: the capture is unusable
};

// Before the gated part of an iteration: its work (the derivatives of the
// current atoms) runs unless the previous trial was rejected, since a
// rejected trial leaves the atoms, their fit fields and so their
// derivatives unchanged (recomputing them would give the same bits).
__global__ void gr_fit_loop_gate_kernel(cudaGraphConditionalHandle gate, const int *hist_acc,
                                        const int *counter, int hist_len) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int c = counter[0];
  unsigned run = 1u;
  if (c > 0 && c <= hist_len) run = hist_acc[c - 1] ? 1u : 0u;
  cudaGraphSetConditional(gate, run);
}

// Stop test after an iteration (the same rule as the host-driven loop):
//   * c >= max_iter iterations done, or
//   * the last max_reject trials were all rejected, or
//   * the last accepted iteration i >= 1 changed the loss by at most
//     tol * |loss before it| (hist[i - 1] -> hist[i]), or
//   * the body ran guard_max times (termination guard).
// Returns 0 (go on) or the reason 1, 2, 3.
__device__ int loop_stop_rule(const double *hist, const int *hist_acc, int c, int hist_len,
                              int max_iter, int max_reject, double tol, bool guard_hit) {
  int stop = (c >= max_iter || guard_hit) ? 1 : 0;
  const int last = (c < hist_len ? c : hist_len) - 1;
  if (!stop && last >= 0) {
    int rejects = 0;
    for (int i = last; i >= 0 && !hist_acc[i]; --i) ++rejects;
    if (rejects >= max_reject) {
      stop = 2;
    } else {
      for (int i = last; i >= 1; --i) {
        if (hist_acc[i]) {
          const double prev = hist[i - 1];
          const double den = fabs(prev) > 1e-300 ? fabs(prev) : 1e-300;
          if (fabs(prev - hist[i]) <= tol * den) stop = 3;
          break;
        }
      }
    }
  }
  return stop;
}

__global__ void gr_fit_loop_stop_kernel(cudaGraphConditionalHandle handle, const double *hist,
                                        const int *hist_acc, const int *counter, int hist_len,
                                        int max_iter, int max_reject, double tol, int *guard,
                                        int guard_max, int *stop_flag) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int runs = guard[0] + 1;
  guard[0] = runs;
  const int stop = loop_stop_rule(hist, hist_acc, counter[0], hist_len, max_iter, max_reject,
                                  tol, runs >= guard_max);
  if (stop_flag) stop_flag[0] = stop;
  cudaGraphSetConditional(handle, stop ? 0u : 1u);
}

// Stop test of a batch: every running problem takes the single-problem test
// on its own history and leaves the batch when it stops; the loop goes on
// while any problem runs (and the guard allows).
__global__ void __launch_bounds__(256)
    gr_batch_stop_kernel(const BatchProb *__restrict__ probs, int n, int *active,
                         cudaGraphConditionalHandle handle, int *guard, int guard_max,
                         int max_reject) {
  __shared__ int runs;
  if (threadIdx.x == 0) {
    runs = guard[0] + 1;
    guard[0] = runs;
  }
  __syncthreads();
  int any = 0;
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    if (!active[p]) continue;
    const BatchProb &B = probs[p];
    if (loop_stop_rule(B.hist, B.hist_acc, *B.counter, B.hist_len, B.max_iter, max_reject,
                       B.tol, runs >= guard_max))
      active[p] = 0;
    else
      any = 1;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) cudaGraphSetConditional(handle, any ? 1u : 0u);
}

int fit_loop_begin(cudaStream_t stream, int *guard, FitLoop **out) {
  if (!out || !guard) return kErrArg;
  *out = nullptr;
  FitLoop *L = new FitLoop();
  L->guard = guard;
  auto fail = [&](int code) {
    if (L->graph) cudaGraphDestroy(L->graph);
    delete L;
    return code;
  };
  if (cudaGraphCreate(&L->graph, 0) != cudaSuccess) return fail(kErrLaunch);
  // every launch: clear the guard, then run the body while the condition is
  // set (it starts at 1: the body runs at least once)
  cudaMemsetParams ms = {};
  ms.dst = guard;
  ms.value = 0;
  ms.elementSize = sizeof(int);
  ms.width = 1;
  ms.height = 1;
  ms.pitch = sizeof(int);
  cudaGraphNode_t clear;
  if (cudaGraphAddMemsetNode(&clear, L->graph, nullptr, 0, &ms) != cudaSuccess)
    return fail(kErrLaunch);
  if (cudaGraphConditionalHandleCreate(&L->handle, L->graph, 1u, cudaGraphCondAssignDefault) !=
      cudaSuccess)
    return fail(kErrLaunch);
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = L->handle;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t loop;
  if (cudaGraphAddNode(&loop, L->graph, &clear, nullptr, 1, &p) != cudaSuccess)
    return fail(kErrLaunch);
  L->body = p.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(stream, L->body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return fail(kErrLaunch);
  L->capturing = true;
  *out = L;
  return kOk;
}

// The nodes that later captured work on stream depends on.
static bool capture_deps(cudaStream_t stream, std::vector<cudaGraphNode_t> &deps) {
  cudaStreamCaptureStatus st;
  const cudaGraphNode_t *d = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(stream, &st, nullptr, nullptr, &d, nullptr, &nd) != cudaSuccess ||
      st != cudaStreamCaptureStatusActive)
    return false;
  deps.assign(d, d + nd);
  return true;
}

// Capture moves into the body of an IF node: a gate kernel (captured into
// the loop body) sets the IF condition each iteration from the accept
// history; the work issued on stream until fit_loop_gate_end is captured
// into the IF node's body.  The capture is ended and restarted around the
// node, so the body graph is never edited while it is being captured into.
int fit_loop_gate_begin(FitLoop *L, cudaStream_t stream, const int *hist_acc, const int *counter,
                        int hist_len) {
  if (!L || !L->capturing || L->gated || L->gate_node) return kErrArg;
  if (!hist_acc || !counter || hist_len < 1) return kErrArg;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  std::vector<cudaGraphNode_t> deps;
  cudaGraph_t g = nullptr;
  bool ok = capture_deps(stream, deps) && cudaStreamEndCapture(stream, &g) == cudaSuccess;
  ok = ok && cudaGraphConditionalHandleCreate(&L->gate, L->body, 1u,
                                              cudaGraphCondAssignDefault) == cudaSuccess;
  ok = ok && cudaStreamBeginCaptureToGraph(stream, L->body, deps.empty() ? nullptr : deps.data(),
                                           nullptr, deps.size(), mode) == cudaSuccess;
  if (ok) {
    gr_fit_loop_gate_kernel<<<1, 32, 0, stream>>>(L->gate, hist_acc, counter, hist_len);
    ok = cudaGetLastError() == cudaSuccess && capture_deps(stream, deps) &&
         cudaStreamEndCapture(stream, &g) == cudaSuccess;
  }
  cudaGraphNodeParams p = {};
  if (ok) {
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = L->gate;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    ok = cudaGraphAddNode(&L->gate_node, L->body, deps.empty() ? nullptr : deps.data(), nullptr,
                          deps.size(), &p) == cudaSuccess;
  }
  ok = ok && cudaStreamBeginCaptureToGraph(stream, p.conditional.phGraph_out[0], nullptr,
                                           nullptr, 0, mode) == cudaSuccess;
  if (!ok) {
    // leave the stream capturing into the loop body so the caller's
    // fit_loop_end still ends the capture (and reports the failure)
    cudaStreamCaptureStatus st;
    if (cudaStreamIsCapturing(stream, &st) != cudaSuccess || st != cudaStreamCaptureStatusActive)
      cudaStreamBeginCaptureToGraph(stream, L->body, nullptr, nullptr, 0, mode);
    L->failed = true;
    return kErrLaunch;
  }
  L->gated = true;
  return kOk;
}

// Capture returns to the loop body, after the IF node.
int fit_loop_gate_end(FitLoop *L, cudaStream_t stream) {
  if (!L || !L->capturing || !L->gated) return kErrArg;
  L->gated = false;
  cudaGraph_t g = nullptr;
  const bool ended = cudaStreamEndCapture(stream, &g) == cudaSuccess;
  const bool ok = ended && cudaStreamBeginCaptureToGraph(stream, L->body, &L->gate_node, nullptr,
                                                         1, cudaStreamCaptureModeThreadLocal) ==
                               cudaSuccess;
  if (!ok) {
    cudaStreamCaptureStatus st;
    if (cudaStreamIsCapturing(stream, &st) != cudaSuccess || st != cudaStreamCaptureStatusActive)
      cudaStreamBeginCaptureToGraph(stream, L->body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal);
    L->failed = true;
    return kErrLaunch;
  }
  return kOk;
}

int fit_loop_end(FitLoop *L, cudaStream_t stream, const double *hist, const int *hist_acc,
                 const int *counter, int hist_len, int max_iter, int max_reject, double tol,
                 int guard_max, int *stop_flag) {
  if (!L || !L->capturing) return kErrArg;
  int rc = L->failed ? kErrLaunch : kOk;
  if (L->gated) {              // a gated part left open: close it, fail the loop
    fit_loop_gate_end(L, stream);
    rc = kErrArg;
  }
  if (!hist || !hist_acc || !counter || hist_len < 1 || max_iter < 1 || max_reject < 1 ||
      guard_max < 1)
    rc = kErrArg;
  if (rc == kOk) {
    gr_fit_loop_stop_kernel<<<1, 32, 0, stream>>>(L->handle, hist, hist_acc, counter, hist_len,
                                                  max_iter, max_reject, tol, L->guard, guard_max,
                                                  stop_flag);
    if (cudaGetLastError() != cudaSuccess) rc = kErrLaunch;
  }
  cudaGraph_t captured = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(stream, &captured);
  L->capturing = false;
  if (ec != cudaSuccess && rc == kOk) rc = kErrLaunch;
  L->captured_ok = rc == kOk;
  return rc;
}

// Instantiation is separate from the capture (it touches no stream).
int fit_loop_instantiate(FitLoop *L) {
  if (!L || L->capturing || !L->captured_ok) return kErrArg;
  if (L->exec) return kOk;
  if (cudaGraphInstantiate(&L->exec, L->graph, 0) != cudaSuccess) {
    L->exec = nullptr;
    return kErrLaunch;
  }
  return kOk;
}

int fit_loop_launch(FitLoop *L, cudaStream_t stream) {
  if (!L || !L->exec || L->capturing) return kErrArg;
  if (cudaGraphLaunch(L->exec, stream) != cudaSuccess) return kErrLaunch;
  note_launches(1);
  return kOk;
}

int fit_loop_destroy(FitLoop *L) {
  if (!L) return kOk;
  if (L->exec) cudaGraphExecDestroy(L->exec);
  if (L->graph) cudaGraphDestroy(L->graph);
  delete L;
  return kOk;
}

// A loop whose captured body sets the WHILE condition itself (a batch's stop
// kernel): end the capture without the single-problem stop test.
int fit_loop_end_open(FitLoop *L, cudaStream_t stream) {
  if (!L || !L->capturing) return kErrArg;
  int rc = L->failed ? kErrLaunch : kOk;
  if (L->gated) {
    fit_loop_gate_end(L, stream);
    rc = kErrArg;
  }
  cudaGraph_t captured = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(stream, &captured);
  L->capturing = false;
  if (ec != cudaSuccess && rc == kOk) rc = kErrLaunch;
  L->captured_ok = rc == kOk;
  return rc;
}

// ---- batches of small 2D fits ---------------------------------------------
// The batch's device tables and buffers live in one caller-owned workspace:
//   tables   problem descriptors, per-kernel block offsets, active flags;
//   clear    the projections' finished-block counters and bitmaps, one
//            contiguous region cleared by one memset per iteration;
//   then per problem the loss partials, pair records and derivative
//   partials.
struct Batch {
  int n = 0, P = 0, max_reject = 8, guard_max = 1;
  BatchLaunch L{};
  void *clear = nullptr;
  size_t clear_bytes = 0;
  std::vector<BatchProb> h_probs;     // host copies of the tables (kept while
  std::vector<int> h_tables;          // their copies may be in flight)
  std::vector<int> h_ones;
};

namespace {

// per-problem shapes fixed by the problem alone
struct BatchShape {
  TileCfg tc;
  int W, items;
  DerivCfg cfg;
  size_t bitmap_bytes, loss_bytes, pair_bytes, part_bytes;
  int blocks[6];   // bin, proj, deriv, fin, solve, acc
};

bool batch_shape(const BatchProb &p, BatchShape &s) {
  const int n = p.cur.n, A = p.g.n_angles, D0 = p.g.ax[0].n;
  if (p.g.K != 1 || n < 1 || A < 1) return false;
  s.tc = make_tiles(1, D0, 1, kTile1D);
  s.W = (n + 31) / 32;
  // the configuration the problem's own 2D projection uses (4 warps, one
  // list entry per thread: W < 8) and its fused loss sum
  if (s.W >= 8) return false;
  s.items = A * s.tc.ntiles;
  if (s.items > 8192) return false;
  s.cfg = deriv_cfg(1, n, A, 2, g_tuning, true);
  if (s.cfg.ch > s.cfg.sg / s.cfg.rs) return false;     // one angle per lane
  s.bitmap_bytes = align_up((size_t)s.items * s.W * sizeof(uint32_t));
  s.loss_bytes = align_up((size_t)s.items * sizeof(double));
  s.pair_bytes = align_up((size_t)A * n * 2 * sizeof(float4));
  s.part_bytes = align_up((size_t)s.cfg.nchunks * s.cfg.qn * n * sizeof(float));
  const int P = p.cur.r_iso ? 4 : 6;
  const long long warps = (long long)((n + s.cfg.ag - 1) / s.cfg.ag) * s.cfg.nchunks;
  s.blocks[0] = ((n + 127) / 128) * A;
  s.blocks[1] = s.items;
  s.blocks[2] = (int)((warps + 3) / 4);
  s.blocks[3] = finalize_blocks(n);
  s.blocks[4] = (n * 8 + 31) / 32;
  const long long acc = ((long long)n * P + 255) / 256;
  s.blocks[5] = (int)(acc < 1 ? 1 : (acc > 152 * 8 ? 152 * 8 : acc));
  return true;
}

size_t batch_table_bytes(int n) {
  return align_up((size_t)n * sizeof(BatchProb)) + align_up(6 * (size_t)(n + 1) * sizeof(int)) +
         align_up((size_t)n * sizeof(int));
}

}  // namespace

size_t batch_workspace_bytes(const BatchProb *probs, int n) {
  if (!probs || n < 1) return 0;
  size_t b = batch_table_bytes(n) + align_up((size_t)n * sizeof(int));
  for (int p = 0; p < n; ++p) {
    BatchShape s;
    if (!batch_shape(probs[p], s)) return 0;
    b += s.bitmap_bytes + s.loss_bytes + s.pair_bytes + s.part_bytes;
  }
  return b;
}

int batch_create(const BatchProb *probs, int n, void *ws, size_t ws_bytes, int max_reject,
                 cudaStream_t stream, Batch **out) {
  if (!out || !probs || n < 1 || !ws || max_reject < 1) return kErrArg;
  *out = nullptr;
  const size_t need = batch_workspace_bytes(probs, n);
  if (need == 0) return kErrArg;
  if (ws_bytes < need) return kErrWorkspace;
  const int P = probs[0].cur.r_iso ? 4 : 6;
  std::vector<BatchShape> sh(n);
  for (int p = 0; p < n; ++p) {
    if (!batch_shape(probs[p], sh[p])) return kErrArg;
    if ((probs[p].cur.r_iso ? 4 : 6) != P || probs[p].trial.r_iso != probs[p].cur.r_iso ||
        probs[p].trial.n != probs[p].cur.n || probs[p].hist_len < 1 || probs[p].max_iter < 1)
      return kErrArg;
  }
  Batch *B = new (std::nothrow) Batch();
  if (!B) return kErrLaunch;
  B->n = n;
  B->P = P;
  B->max_reject = max_reject;
  char *base = static_cast<char *>(ws);
  char *tables = base;
  char *w = base + batch_table_bytes(n);
  B->clear = w;
  int *done = reinterpret_cast<int *>(w);
  w += align_up((size_t)n * sizeof(int));
  B->h_probs.assign(probs, probs + n);
  int max_iter = 1;
  for (int p = 0; p < n; ++p) {
    BatchProb &q = B->h_probs[p];
    const BatchShape &s = sh[p];
    q.tc = s.tc;
    q.W = s.W;
    q.items = s.items;
    q.cfg = s.cfg;
    q.bitmap = reinterpret_cast<uint32_t *>(w);
    w += s.bitmap_bytes;
    q.done = done + p;
    q.P = P;
    q.pr = P == 4 ? 1 : 3;
    if (q.max_iter > max_iter) max_iter = q.max_iter;
  }
  B->clear_bytes = (size_t)(w - static_cast<char *>(B->clear));
  for (int p = 0; p < n; ++p) {
    BatchProb &q = B->h_probs[p];
    const BatchShape &s = sh[p];
    double *loss_part = reinterpret_cast<double *>(w);
    w += s.loss_bytes;
    q.pairs = reinterpret_cast<float4 *>(w);
    w += s.pair_bytes;
    q.part = reinterpret_cast<float *>(w);
    w += s.part_bytes;
    q.out.R = nullptr;
    q.out.epilogue = kEpiL2;
    q.out.bg = 0.f;
    q.out.beta = nullptr;
    q.out.loss_part = loss_part;
    q.out.psf = 0;
    q.din.mode = kModeField;
    q.din.order = 2;
    q.din.alpha = q.out.alpha;
    q.din.beta = nullptr;
    q.din.beta_const = 1.f;
    q.din.psf = 0;
  }
  // tables: descriptors, offsets (bin, proj, deriv, fin, solve, acc), active
  BatchProb *d_probs = reinterpret_cast<BatchProb *>(tables);
  int *d_off = reinterpret_cast<int *>(tables + align_up((size_t)n * sizeof(BatchProb)));
  int *d_active = reinterpret_cast<int *>(tables + align_up((size_t)n * sizeof(BatchProb)) +
                                          align_up(6 * (size_t)(n + 1) * sizeof(int)));
  B->h_tables.assign(6 * (size_t)(n + 1), 0);
  int grid[6];
  for (int k = 0; k < 6; ++k) {
    long long acc = 0;
    for (int p = 0; p < n; ++p) {
      B->h_tables[(size_t)k * (n + 1) + p] = (int)acc;
      acc += sh[p].blocks[k];
    }
    B->h_tables[(size_t)k * (n + 1) + n] = (int)acc;
    if (acc > 0x7fffffffLL) {
      delete B;
      return kErrArg;
    }
    grid[k] = (int)acc;
  }
  B->h_ones.assign(n, 1);
  B->guard_max = max_iter + max_reject + 2;
  B->L.probs = d_probs;
  B->L.n = n;
  B->L.active = d_active;
  B->L.off_bin = d_off;
  B->L.off_proj = d_off + (n + 1);
  B->L.off_deriv = d_off + 2 * (n + 1);
  B->L.off_fin = d_off + 3 * (n + 1);
  B->L.off_solve = d_off + 4 * (n + 1);
  B->L.off_acc = d_off + 5 * (n + 1);
  B->L.grid_bin = grid[0];
  B->L.grid_proj = grid[1];
  B->L.grid_deriv = grid[2];
  B->L.grid_fin = grid[3];
  B->L.grid_solve = grid[4];
  B->L.grid_acc = grid[5];
  if (cudaMemcpyAsync(d_probs, B->h_probs.data(), (size_t)n * sizeof(BatchProb),
                      cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaMemcpyAsync(d_off, B->h_tables.data(), B->h_tables.size() * sizeof(int),
                      cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess) {
    delete B;
    return kErrLaunch;
  }
  *out = B;
  return kOk;
}

// Before each launch of the batch's loop: every problem active, the fit
// fields and loss of its current atoms (the problems' own prologue).
int batch_prologue(Batch *B, cudaStream_t stream) {
  if (!B) return kErrArg;
  if (cudaMemcpyAsync(B->L.active, B->h_ones.data(), (size_t)B->n * sizeof(int),
                      cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaMemsetAsync(B->clear, 0, B->clear_bytes, stream) != cudaSuccess)
    return kErrLaunch;
  int rc = launch_batch_bin(B->L, 0, stream);
  if (rc == kOk) rc = launch_batch_project(B->L, 0, stream);
  return rc;
}

// One iteration of every running problem (the body of the batch's loop):
// derivatives (after an accepted trial), FP64 block solves, trial
// projection, accept, then the batch stop test, which sets the loop's WHILE
// condition.
int batch_iterate(Batch *B, FitLoop *L, cudaStream_t stream) {
  if (!B || !L || !L->capturing) return kErrArg;
  int rc = launch_batch_derivs(B->L, stream);
  if (rc == kOk) rc = launch_batch_solve(B->L, B->P, stream);
  if (rc == kOk && cudaMemsetAsync(B->clear, 0, B->clear_bytes, stream) != cudaSuccess)
    rc = kErrLaunch;
  if (rc == kOk) rc = launch_batch_bin(B->L, 1, stream);
  if (rc == kOk) rc = launch_batch_project(B->L, 1, stream);
  if (rc == kOk) rc = launch_batch_accept(B->L, stream);
  if (rc == kOk) {
    gr_batch_stop_kernel<<<1, 256, 0, stream>>>(B->L.probs, B->n, B->L.active, L->handle,
                                                 L->guard, B->guard_max, B->max_reject);
    note_launches(1);
    if (cudaGetLastError() != cudaSuccess) rc = kErrLaunch;
  }
  if (rc != kOk) L->failed = true;
  return rc;
}

void batch_destroy(Batch *B) { delete B; }

int preload_loop() {
  return preload_fn(gr_fit_loop_stop_kernel) + preload_fn(gr_fit_loop_gate_kernel) +
         preload_fn(gr_batch_stop_kernel);
}

}  // namespace gr

extern "C" {

int gr_fit_loop_begin(void *stream, int *guard, void **loop) {
  gr::FitLoop *L = nullptr;
  const int rc = gr::fit_loop_begin(static_cast<cudaStream_t>(stream), guard, &L);
  if (loop) *loop = L;
  return rc;
}

int gr_fit_loop_end(void *loop, void *stream, const double *hist, const int *hist_acc,
                    const int *counter, int hist_len, int max_iter, int max_reject, double tol,
                    int guard_max, int *stop_flag) {
  return gr::fit_loop_end(static_cast<gr::FitLoop *>(loop), static_cast<cudaStream_t>(stream),
                          hist, hist_acc, counter, hist_len, max_iter, max_reject, tol, guard_max,
                          stop_flag);
}

int gr_fit_loop_gate_begin(void *loop, void *stream, const int *hist_acc, const int *counter,
                           int hist_len) {
  return gr::fit_loop_gate_begin(static_cast<gr::FitLoop *>(loop),
                                 static_cast<cudaStream_t>(stream), hist_acc, counter, hist_len);
}

int gr_fit_loop_gate_end(void *loop, void *stream) {
  return gr::fit_loop_gate_end(static_cast<gr::FitLoop *>(loop),
                               static_cast<cudaStream_t>(stream));
}

int gr_fit_loop_instantiate(void *loop) {
  return gr::fit_loop_instantiate(static_cast<gr::FitLoop *>(loop));
}

int gr_fit_loop_launch(void *loop, void *stream) {
  return gr::fit_loop_launch(static_cast<gr::FitLoop *>(loop), static_cast<cudaStream_t>(stream));
}

int gr_fit_loop_destroy(void *loop) {
  return gr::fit_loop_destroy(static_cast<gr::FitLoop *>(loop));
}

int gr_fit_loop_end_open(void *loop, void *stream) {
  return gr::fit_loop_end_open(static_cast<gr::FitLoop *>(loop),
                               static_cast<cudaStream_t>(stream));
}

int gr_batch_prologue(void *batch, void *stream) {
  return gr::batch_prologue(static_cast<gr::Batch *>(batch), static_cast<cudaStream_t>(stream));
}

int gr_batch_iterate(void *batch, void *loop, void *stream) {
  return gr::batch_iterate(static_cast<gr::Batch *>(batch), static_cast<gr::FitLoop *>(loop),
                           static_cast<cudaStream_t>(stream));
}

int gr_batch_destroy(void *batch) {
  gr::batch_destroy(static_cast<gr::Batch *>(batch));
  return 0;
}

}  // extern "C"
