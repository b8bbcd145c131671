"""Served batch fitting: a continuous-batching request loop on one GPU.

Fitting requests of uneven size (2D or 3D, any atom count, angle count and
detector size) arrive over time.  The server admits a request as soon as a
slot and enough free HBM are available, also while other requests are being
fitted; every admitted request owns its device buffers and a CUDA stream, and
one damped-Newton iteration

  gr_atom_derivs(all atoms)      -> gradient and Hessian blocks
  gr_newton_solve                -> trial parameters (FP64 solves on the device)
  gr_fit_forward(trial atoms)    -> trial fit fields, trial loss
  gr_newton_accept               -> device-side accept/reject, damping update,
                                    loss history
  gr_accept_fields               -> an accepted trial's fields become current

(one projection per iteration: the current atoms' fields come from the
prologue's gr_fit_forward, an accepted trial, or stay after a rejection)

is captured once into the body of a device-resident loop (engine.FitLoop: a
CUDA graph whose WHILE node repeats the iteration until a device-side stop
test ends it: relative loss change below ``tol`` after an accepted step,
``max_iter`` iterations, or 8 rejected trials in a row).  A whole fit is one
graph launch; the host only polls a completion event and reads the result.
Requests on different streams overlap on the device.  Where the device loop
cannot be built, the request falls back to a graph of one iteration replayed
a few iterations at a time, with the same stop test on the host copy of the
loss history.  A request's result does not depend on what else is running:
its kernels are deterministic and its state private (tests/test_serving_gpu.py
checks that results alone and in the mix agree).

Host-side care that keeps the loop from stalling behind fits in flight:
buffers of a new request are built on a separate setup stream; finished
loop graphs are destroyed only when no fit runs (destroying an executable
graph waits for the device to idle); pinned host buffers are pooled.  Among
requests that have arrived, the largest are admitted first, so the longest
fits start early.

The process should give every stream its own hardware work queue
(environment ``CUDA_DEVICE_MAX_CONNECTIONS`` >= n_streams + 1, set before CUDA
starts): with fewer, streams share queues and a request's set-up can wait
behind another request's whole fit.

``serve_plain`` is the baseline: the same fits one after another with the
eager host-driven loop, one host sync per iteration.
"""
import collections
import time

import numpy as np
import torch

from . import _lib, engine
from .geometry import DeviceGeometry

MAX_BACKTRACK = 8


class FitRequest:
    """One fitting problem.  ``make_data(geom, device, stream)`` returns the
    data sinogram as a float32 device tensor (called at admission) unless the
    request carries it as ``data_host`` (pinned host memory), which admission
    copies in."""

    def device_data(self, geom, device, stream):
        """The data sinogram on the device: the carried payload copied in
        (asynchronously on ``stream``), else ``make_data``."""
        if self.data_host is not None:
            d = torch.empty(geom.shape, dtype=torch.float32, device=device)
            with torch.cuda.stream(stream):
                d.copy_(self.data_host.reshape(geom.shape), non_blocking=True)
            return d
        return self.make_data(geom, device, stream)

    def __init__(self, rid, orientations, ortho, detector, init, make_data, fit="l2",
                 background=0.0, max_iter=100, tol=1e-6, arrival=0.0, lam0=1.0):
        self.id = rid
        self.orientations = orientations
        self.ortho = ortho
        self.detector = detector
        self.init = init
        self.make_data = make_data
        self.fit = fit
        self.background = background
        self.max_iter = max_iter
        self.tol = tol
        self.arrival = arrival
        self.lam0 = lam0
        self.data_host = None       # optional payload (pinned host tensor)
        n = len(init[0])
        cells = len(orientations) * int(np.prod([len(d) for d in detector]))
        self.size_hint = (n, cells)


class _Slot:
    """Device state of one admitted request."""

    def __init__(self, req, stream, device, use_graph=True, iters_per_launch=4,
                 device_loop=True, setup_stream=None, pinned=None):
        self.req = req
        self.stream = stream
        self.dev = device
        self.k = iters_per_launch
        # Buffers are built and filled on a setup stream: the compute stream
        # may still hold queued fits of earlier requests.
        setup = setup_stream if setup_stream is not None else stream
        t_start = time.perf_counter()
        with torch.cuda.stream(setup):
            self.geom = DeviceGeometry(req.orientations, req.ortho, req.detector, device)
            I0, x0, r0 = req.init
            n = len(I0)
            self.cur = engine.DeviceAtoms(I0, x0, r0, device)
            self.trial = engine.DeviceAtoms(I0, x0, r0, device)
            self.dim, self.iso = self.cur.dim, self.cur.iso
            self.P = self.cur.n_params()
            self.theta = torch.cat([self.cur.I.double().reshape(-1, 1), self.cur.x.double(),
                                    self.cur.r.double().reshape(n, -1)], 1).contiguous()
            self.theta_trial = self.theta.clone()
            self.lam = torch.full((n,), float(req.lam0), dtype=torch.float64, device=device)
            shape = self.geom.shape
            self.data = req.device_data(self.geom, device, setup)
            self.alpha = torch.empty(shape, dtype=torch.float32, device=device)
            self.beta = (torch.empty(shape, dtype=torch.float32, device=device)
                         if req.fit == "kl" else None)
            # the trial's fit fields (adopted when the trial is accepted)
            self.alpha_t = torch.empty(shape, dtype=torch.float32, device=device)
            self.beta_t = (torch.empty(shape, dtype=torch.float32, device=device)
                           if req.fit == "kl" else None)
            self.loss_cur = torch.zeros((), dtype=torch.float64, device=device)
            self.loss_trial = torch.zeros((), dtype=torch.float64, device=device)
            self.f = torch.empty(n, dtype=torch.float64, device=device)
            self.g = torch.empty((n, self.P), dtype=torch.float64, device=device)
            self.H = torch.empty((n, self.P, self.P), dtype=torch.float64, device=device)
            self.step = torch.empty(n, dtype=torch.float64, device=device)
            self.ws_p = torch.empty(max(256, engine.workspace_bytes(_lib.GR_OP_PROJECT, self.cur, self.geom)),
                                    dtype=torch.uint8, device=device)
            self.ws_d = torch.empty(max(256, engine.workspace_bytes(_lib.GR_OP_DERIVS_2, self.cur, self.geom)),
                                    dtype=torch.uint8, device=device)
            L = req.max_iter + MAX_BACKTRACK + 8
            self.hist = torch.zeros(L, dtype=torch.float64, device=device)
            self.hist_acc = torch.zeros(L, dtype=torch.int32, device=device)
            self.counter = torch.zeros(1, dtype=torch.int32, device=device)
            if pinned is None:
                pinned = (torch.zeros(L, dtype=torch.float64).pin_memory(),
                          torch.zeros(L, dtype=torch.int32).pin_memory(),
                          torch.zeros(1, dtype=torch.int32).pin_memory())
            self.pinned = pinned
            self.h_hist, self.h_acc, self.h_counter = pinned
        t_bufs = time.perf_counter()
        if setup is not stream:
            ready = torch.cuda.Event()
            ready.record(setup)
            stream.wait_event(ready)
            for t in (self.geom.frames, self.geom.det, self.cur.I, self.cur.x,
                      self.cur.r, self.trial.I, self.trial.x, self.trial.r, self.theta,
                      self.theta_trial, self.lam, self.data, self.alpha, self.beta,
                      self.alpha_t, self.beta_t,
                      self.loss_cur, self.loss_trial, self.f, self.g, self.H, self.step,
                      self.ws_p, self.ws_d, self.hist, self.hist_acc, self.counter):
                for u in (t if isinstance(t, (list, tuple)) else (t,)):
                    if u is not None:
                        u.record_stream(stream)
        t_cap = time.perf_counter()
        with torch.cuda.stream(stream):
            self.event = torch.cuda.Event()
            self.graph = None
            self.loop = None
            self.loss0 = None
            if use_graph and device_loop:
                # the whole fit as one graph: the iteration repeats on the
                # device until the device-side stop test ends it
                try:
                    self.loop = engine.FitLoop(stream, self.iterate, self.hist, self.hist_acc,
                                               self.counter, req.max_iter, MAX_BACKTRACK,
                                               req.tol, device)
                except _lib.EngineError:
                    self.loop = None
            t_loop = time.perf_counter()
            self.phase_seconds = {"buffers": t_bufs - t_start, "streams": t_cap - t_bufs,
                                  "capture": t_loop - t_cap}
            if self.loop is not None:
                self.iterations_launched = 0
                return
            self.prologue()
            self.iterate()                       # eager first iteration (also warms up)
            if use_graph:
                # captured directly on this request's stream: the
                # torch.cuda.graph context would synchronise the whole device
                # and run the garbage collector at every admission, stalling
                # the requests already in flight (no allocation happens
                # inside the capture: every buffer exists already)
                self.graph = torch.cuda.CUDAGraph()
                self.graph.capture_begin(capture_error_mode="thread_local")
                try:
                    self.iterate()
                finally:
                    self.graph.capture_end()
            self._copy_back()
        self.iterations_launched = 1

    def bytes(self):
        tensors = [self.data, self.alpha, self.beta, self.alpha_t, self.beta_t, self.g,
                   self.H, self.ws_p, self.ws_d,
                   self.theta, self.theta_trial]
        return sum(t.numel() * t.element_size() for t in tensors if t is not None)

    def prologue(self):
        """Fit fields and loss of the starting atoms (once per fit)."""
        r = self.req
        engine.fit_forward_into(self.cur, self.geom, self.data, r.fit, r.background, None,
                                self.alpha, self.beta, self.loss_cur, self.ws_p)

    def iterate(self):
        """One damped-Newton iteration.  The current atoms' fields are always
        valid here (from the prologue, an accepted trial, or unchanged after
        a rejected one), so only the trial is projected."""
        r = self.req
        beta_c = 1.0 if r.fit == "l2" else 0.0
        engine.atom_derivs_into(self.cur, self.geom, "field", self.alpha, self.beta, beta_c, 2,
                                self.f, self.g, self.H, self.ws_d)
        engine.newton_solve_into(self.dim, self.iso, self.g, self.H, self.lam, self.theta,
                                 self.theta_trial, self.step, self.trial, self.dev)
        engine.fit_forward_into(self.trial, self.geom, self.data, r.fit, r.background, None,
                                self.alpha_t, self.beta_t, self.loss_trial, self.ws_p)
        engine.newton_accept_into(self.dim, self.iso, self.loss_cur, self.loss_trial,
                                  self.theta, self.theta_trial, self.lam, 1e-4, 1e4,
                                  self.cur, self.trial, self.hist, self.hist_acc,
                                  self.counter, self.dev)
        engine.accept_fields_into(self.loss_cur, self.loss_trial, self.alpha_t, self.alpha,
                                  self.beta_t, self.beta, self.dev)

    def _copy_back(self):
        self.h_counter.copy_(self.counter, non_blocking=True)
        self.h_hist.copy_(self.hist, non_blocking=True)
        self.h_acc.copy_(self.hist_acc, non_blocking=True)
        self.event.record(self.stream)

    def launch(self):
        if self.loop is not None:
            with torch.cuda.stream(self.stream):
                self.prologue()
                self.loop.launch()
                self._copy_back()
            self.iterations_launched = self.req.max_iter
            return
        with torch.cuda.stream(self.stream):
            for _ in range(self.k):
                if self.graph is not None:
                    self.graph.replay()
                else:
                    self.iterate()
            self._copy_back()
        self.iterations_launched += self.k

    def done(self):
        """Convergence test on the host copy of the history (call after the
        event completed).  A device loop has stopped by itself."""
        if self.loop is not None:
            return True
        c = int(self.h_counter[0])
        if c >= self.req.max_iter:
            return True
        hist = self.h_hist.numpy()
        acc = self.h_acc.numpy()
        rejects = 0
        for i in range(c - 1, -1, -1):
            if acc[i]:
                break
            rejects += 1
        if rejects >= MAX_BACKTRACK:
            return True
        # last accepted step
        for i in range(c - 1, 0, -1):
            if acc[i]:
                prev = hist[i - 1]
                return abs(prev - hist[i]) <= self.req.tol * max(abs(prev), 1e-300)
        return False

    def result(self):
        self.stream.synchronize()
        c = int(self.h_counter[0])
        with torch.cuda.stream(self.stream):
            theta = self.theta.cpu().numpy()
            loss = float(self.loss_cur.item())
        return {"theta": theta, "loss": loss, "iterations": min(c, self.req.max_iter)}


_warmed = set()


def _warm_engine(device):
    """Run every kernel family once eagerly on tiny 2D and 3D problems, so
    that the library's one-time per-device set-up happens outside any stream
    capture."""
    if device in _warmed:
        return
    for dim in (2, 3):
        th = np.linspace(0, 3, 3)
        T = np.stack([np.cos(th), np.sin(th)], 1)
        w = (np.stack([-T[:, 1], T[:, 0]], 1),)
        c = np.linspace(-1, 1, 16)
        if dim == 2:
            geom = DeviceGeometry(T, w, [c], device)
            r = np.array([[5.0, 5.0, 0.0]])
        else:
            geom = DeviceGeometry(T, w, [c, c.copy()], device)
            r = np.array([[5.0, 5.0, 5.0, 0.0, 0.0, 0.0]])
        atoms = engine.DeviceAtoms(np.ones(1), np.zeros((1, dim)), r, device)
        data = torch.zeros(geom.shape, dtype=torch.float32, device=device)
        for fit in ("l2", "kl"):
            fw = engine.fit_forward(atoms, geom, data, fit, 1.0)
            engine.atom_derivs(atoms, geom, "field", fw["alpha"], fw["beta"],
                               1.0 if fit == "l2" else 0.0, 2)
    torch.cuda.synchronize(device)
    _warmed.add(device)


class GaussFitServer:
    """Continuous-batching fitting server (see the module docstring)."""

    def __init__(self, device=None, max_slots=32, n_streams=16, hbm_budget=None,
                 hbm_reserve=4 << 30, use_graphs=True, iters_per_launch=4, device_loop=True,
                 largest_first=True):
        self.dev = torch.device(device or "cuda")
        engine._require_cuda(self.dev)
        self.max_slots = max_slots
        self.streams = [torch.cuda.Stream(self.dev) for _ in range(n_streams)]
        self.setup_stream = torch.cuda.Stream(self.dev)
        free, _total = torch.cuda.mem_get_info(self.dev)
        self.budget = hbm_budget if hbm_budget is not None else max(0, free - hbm_reserve)
        self.use_graphs = use_graphs
        self.k = iters_per_launch
        self.device_loop = device_loop
        self.largest_first = largest_first
        self.pending = collections.deque()
        self.active = []
        self.results = {}
        self.in_use = 0
        self.stream_busy = [0] * n_streams
        self.admitted_while_busy = 0
        self.admit_seconds = 0.0     # host time spent setting up admitted requests
        self.admit_phases = {}       # the same by phase (buffers, streams, capture)
        self.device_loops = 0        # requests run as one device-resident loop graph
        # Finished requests' loop graphs are destroyed only when no fit runs:
        # destroying an executable graph waits for the whole device to idle,
        # which would stall the host loop behind every fit in flight.
        self._retired_loops = []
        self._pinned = {}            # history length -> free pinned host buffers
        _warm_engine(self.dev)

    @staticmethod
    def estimate_bytes(req):
        """Upper estimate of a request's device memory (bytes)."""
        n, cells = req.size_hint
        dim = len(req.init[1][0]) if n else 2
        P = 1 + dim + (1 if np.asarray(req.init[2]).reshape(n, -1).shape[1] == 1 else (3 if dim == 2 else 6))
        sino = cells * 4 * (3 + (2 if req.fit == "kl" else 0))
        tiles = max(1, cells // (32 if dim == 2 else 1024)) + len(req.orientations)
        bitmap = tiles * ((n + 31) // 32) * 4 + tiles * 8
        qn = 1 + P + P * (P + 1) // 2
        deriv = 4096 * 32 * qn * 4 + qn * n * 8 + n * qn * 4 * 256
        per_atom = n * (P * P + 4 * P + 16) * 8
        return int(1.3 * (sino + bitmap + deriv + per_atom)) + (8 << 20)

    def submit(self, req):
        self.pending.append(req)

    def _admit(self, now):
        if self.largest_first and len(self.pending) > 1:
            # among the requests that have arrived, the largest go first, so
            # the longest fits start early (arrival order otherwise kept)
            arrived = [r for r in self.pending if r.arrival <= now]
            if len(arrived) > 1:
                later = [r for r in self.pending if r.arrival > now]
                arrived.sort(key=lambda r: -(r.size_hint[0] * r.size_hint[1]))
                self.pending = collections.deque(arrived + later)
        while self.pending and len(self.active) < self.max_slots:
            req = self.pending[0]
            if req.arrival > now:
                break
            need = self.estimate_bytes(req)
            if self.in_use + need > self.budget:
                if not self.active:
                    raise MemoryError("request %s needs %d bytes, budget %d"
                                      % (req.id, need, self.budget))
                break
            self.pending.popleft()
            si = int(np.argmin(self.stream_busy))
            self.stream_busy[si] += 1
            if self.active:
                self.admitted_while_busy += 1
            ta = time.perf_counter()
            L = req.max_iter + MAX_BACKTRACK + 8
            free = self._pinned.get(L)
            slot = _Slot(req, self.streams[si], self.dev, self.use_graphs, self.k,
                         self.device_loop, self.setup_stream, free.pop() if free else None)
            self.admit_seconds += time.perf_counter() - ta
            phases = dict(slot.phase_seconds)
            if slot.loop is not None:
                phases.update(slot.loop.seconds)
            for k, v in phases.items():
                self.admit_phases[k] = self.admit_phases.get(k, 0.0) + v
            slot.stream_index = si
            if slot.loop is not None:
                self.device_loops += 1
            slot.need = need
            slot.t_admit = time.perf_counter()
            self.in_use += need
            self.active.append(slot)
            slot.launch()

    def run(self, t0=None, on_done=None):
        """Serve until every submitted request is finished.  Arrival times
        are seconds after t0 (default: now).  Returns {id: result}."""
        t0 = time.perf_counter() if t0 is None else t0
        while self.pending or self.active:
            now = time.perf_counter() - t0
            self._admit(now)
            progressed = False
            for slot in list(self.active):
                if not slot.event.query():
                    continue
                progressed = True
                if slot.done():
                    res = slot.result()
                    res["arrival"] = slot.req.arrival
                    res["finish"] = time.perf_counter() - t0
                    res["latency"] = res["finish"] - slot.req.arrival
                    self.results[slot.req.id] = res
                    self.active.remove(slot)
                    self.in_use -= slot.need
                    self.stream_busy[slot.stream_index] -= 1
                    if slot.loop is not None:
                        self._retired_loops.append(slot.loop)
                        slot.loop = None
                    self._pinned.setdefault(len(slot.h_hist), []).append(slot.pinned)
                    if on_done:
                        on_done(slot.req, res)
                    del slot
                    if not self.active:
                        self._release_loops()
                else:
                    slot.launch()
            if not progressed:
                if self.pending and not self.active:
                    wait = self.pending[0].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                else:
                    time.sleep(20e-6)
        self._release_loops()
        return self.results

    def _release_loops(self):
        """Destroy the retired loop graphs (nothing of this server runs)."""
        if self._retired_loops:
            torch.cuda.synchronize(self.dev)
            for lp in self._retired_loops:
                lp.close()
            self._retired_loops = []


def serve_plain(requests, device=None, t0=None):
    """Baseline: the same fits one at a time with the eager host-driven loop
    (no graphs, no overlap); a request starts at max(arrival, previous end)."""
    from . import solvers
    dev = torch.device(device or "cuda")
    t0 = time.perf_counter() if t0 is None else t0
    out = {}
    stream = torch.cuda.current_stream(dev)
    for req in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if req.arrival > now:
            time.sleep(req.arrival - now)
        geom = DeviceGeometry(req.orientations, req.ortho, req.detector, dev)
        data = req.device_data(geom, dev, stream)
        atoms = engine.DeviceAtoms(*req.init, dev)
        losses = []
        cur, losses = _plain_fit(atoms, geom, data, req)
        torch.cuda.synchronize(dev)
        fin = time.perf_counter() - t0
        out[req.id] = {"loss": losses[-1], "iterations": len(losses) - 1,
                       "arrival": req.arrival, "finish": fin, "latency": fin - req.arrival}
    return out


def _plain_fit(atoms, geom, data, req):
    """Eager damped Newton with the same accept rule and stopping test."""
    from . import solvers
    dim, iso = atoms.dim, atoms.iso
    theta = solvers.theta_of(atoms.I, atoms.x, atoms.r)
    fit, bg = req.fit, req.background
    beta_c = 1.0 if fit == "l2" else 0.0
    lam = torch.full((atoms.n,), float(req.lam0), dtype=torch.float64, device=geom.device)
    cur = atoms
    losses = []
    rejects = 0
    for it in range(req.max_iter):
        fw = engine.fit_forward(cur, geom, data, fit, bg)
        loss = float(fw["loss"].item())
        if not losses:
            losses.append(loss)
        _f, g, H = engine.atom_derivs(cur, geom, "field", fw["alpha"], fw["beta"], beta_c, 2)
        th, _s, _fl = engine.newton_solve(dim, iso, g.contiguous(), H.contiguous(), lam, theta)
        trial = solvers.atoms_of(th, dim, geom.device)
        new = float(engine.fit_forward(trial, geom, data, fit, bg, want_fields=False)["loss"].item())
        if new <= loss:
            theta, cur = th, trial
            lam = torch.clamp(lam / 2, 1e-4, 1e4)
            losses.append(new)
            rejects = 0
            if abs(loss - new) <= req.tol * max(abs(loss), 1e-300):
                break
        else:
            lam = torch.clamp(lam * 10, 1e-4, 1e4)
            rejects += 1
            if rejects >= MAX_BACKTRACK:
                break
    return cur, losses
