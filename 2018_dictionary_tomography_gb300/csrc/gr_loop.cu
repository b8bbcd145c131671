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
__global__ void gr_fit_loop_stop_kernel(cudaGraphConditionalHandle handle, const double *hist,
                                        const int *hist_acc, const int *counter, int hist_len,
                                        int max_iter, int max_reject, double tol, int *guard,
                                        int guard_max, int *stop_flag) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int runs = guard[0] + 1;
  guard[0] = runs;
  const int c = counter[0];
  int stop = (c >= max_iter || runs >= guard_max) ? 1 : 0;
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
  if (stop_flag) stop_flag[0] = stop;
  cudaGraphSetConditional(handle, stop ? 0u : 1u);
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

int preload_loop() {
  return preload_fn(gr_fit_loop_stop_kernel) + preload_fn(gr_fit_loop_gate_kernel);
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

}  // extern "C"
