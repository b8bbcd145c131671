"""Served batch fitting: a continuous-batching request loop on one GPU.

Fitting requests of uneven size (2D or 3D, any atom count, angle count and
detector size) arrive over time.  The server admits a request as soon as a
slot and enough free HBM are available, also while other requests are being
fitted; every admitted request owns its device buffers and a CUDA stream, and
one damped-Newton iteration

  gr_atom_derivs(all atoms)      -> gradient and Hessian blocks
  gr_newton_solve                -> trial parameters (FP64 block solves)
  gr_fit_forward(trial atoms)    -> trial fit fields, trial loss
  gr_newton_accept               -> device-side accept/reject, damping update,
                                    loss history

(one projection per iteration: the current atoms' fields come from the
prologue's gr_fit_forward or an accepted trial; the derivatives read them
only right after one of those, while they are still in the trial buffers,
so they are never copied)

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
graph waits for the device to idle); pinned host buffers are pooled.  Requests
are admitted in arrival order, except that while fewer than half the streams
have a fit in flight the largest arrived request goes first
(``largest_first="when_idle"``, the default): a server starting on a full
queue otherwise spends its first tens of milliseconds setting up small fits
that finish at once while the device idles (512 requests submitted at once:
1.494 s against 1.503 s in arrival order).  ``largest_first=True`` sorts
every admission by size and "both_ends" alternates the largest and the
smallest; both leave the small fits, whose time is mostly host set-up, to the
end.  A request is admitted only onto a stream with no fit in
flight (``exclusive_streams``): a stream runs its work in order, and a
whole fit is one graph launch, so a request queued behind another on the
same stream would wait for that entire fit however little work it has.

3D fits skip the (angle, tile) items of their forwards that no atom meets
(``skip_empty``, engine.fit_forward_into(empty_loss=...)): bitwise the same
fits, 26 % less 3D projection time on the stream's requests.

With ``batch_max`` > 1, small 2D fits (up to 224 atoms, L2, no regulariser)
that are admitted together run as one batched device loop
(``engine.BatchLoop``): every kernel of an iteration is one launch over a
table of the fits, each fit leaves the batch at its own stop test, and every
fit ends bitwise where its own loop would (tests/test_serving_gpu.py).  It
is off by default: the batch's kernels cover its stopped members' blocks and
its loop runs until its last member stops, which costs more device time
(the stream's 155 batchable fits: 0.100 s batched against 0.079 s in their
own loops) than the host set-up it saves (admission 0.48 -> 0.38 s), and the
mix is bound by device work (512 requests: 1.537 s with batches of 8 against
1.494 s without).

The process should give every stream its own hardware work queue
(environment ``CUDA_DEVICE_MAX_CONNECTIONS`` >= n_streams + 1, at most 32,
set before CUDA starts): streams that share a queue are serialised the same
way.

``serve_plain`` is the baseline: the same fits one after another with the
eager host-driven loop, one host sync per iteration.
"""
import collections
import contextlib
import math
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
                 background=0.0, max_iter=100, tol=1e-6, arrival=0.0, lam0=1.0,
                 lam_max=1e8, reg=None):
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
        # damping bounds of the all-atoms step: lam in [1e-4, lam_max].  The
        # reference clamps its per-atom damping at 1e4 (NewtonGaussian.py:92);
        # all atoms stepping at once need more: the steps of overlapping
        # atoms add up, and with the ceiling at 1e4 the backtracking stalls
        # there, repeating one rejected trial (on the 512-request stream 204
        # fits ended without an accepted step; with 1e8 none)
        self.lam_max = lam_max
        # optional regulariser (a regularisation.Joubert/Mass/Volume/Radius/Iso):
        # its value joins the fit's loss and its gradient and Hessian the
        # blocks, as in the reference's Newton loop (NewtonGaussian.py:59-66)
        self.reg = reg
        self.data_host = None       # optional payload (pinned host tensor)
        n = len(init[0])
        cells = len(orientations) * int(np.prod([len(d) for d in detector]))
        self.size_hint = (n, cells)


def validate_request(req):
    """Host-side checks of a request before it may queue: consistent shapes
    (orientations (A, d) with ortho/detector for a 2D, 2.5D or 3D geometry;
    atoms I (N,), x (N, dim), r (N, 1 | 3 | 6)), at least one atom and one
    angle, finite parameters and payload, a known fit with a positive KL
    background, max_iter >= 1 and tol >= 0.  Raises ValueError naming the
    first problem found."""
    T = np.asarray(req.orientations, dtype=np.float64)
    if T.ndim != 2 or T.shape[0] < 1 or T.shape[1] not in (2, 3):
        raise ValueError("request %s: orientations must be (A, 2|3) with A >= 1" % req.id)
    A, dT = T.shape
    det = [np.asarray(d, dtype=np.float64).reshape(-1) for d in req.detector]
    if len(det) not in (1, 2) or any(d.size < 1 for d in det):
        raise ValueError("request %s: one or two non-empty detector coordinate vectors" % req.id)
    if dT == 3 and len(det) != 2:
        raise ValueError("request %s: 3D orientations need two detector axes" % req.id)
    ortho = [np.asarray(o, dtype=np.float64) for o in req.ortho]
    n_axes = len(det) if dT == 3 else 1
    if len(ortho) < n_axes or any(o.shape != (A, dT) for o in ortho[:n_axes]):
        raise ValueError("request %s: ortho must hold %d arrays of shape (%d, %d)"
                         % (req.id, n_axes, A, dT))
    dim = 3 if (dT == 3 or len(det) == 2) else 2
    I, x, r = (np.asarray(v, dtype=np.float64) for v in req.init)
    n = I.size
    if n < 1:
        raise ValueError("request %s: no atoms" % req.id)
    if x.size != n * dim:
        raise ValueError("request %s: x must be (%d, %d)" % (req.id, n, dim))
    pr = r.size // n if r.size % n == 0 else -1
    if pr not in (1, 3 if dim == 2 else 6):
        raise ValueError("request %s: r must be (%d, 1) or (%d, %d)"
                         % (req.id, n, n, 3 if dim == 2 else 6))
    for name, v in (("I", I), ("x", x), ("r", r), ("orientations", T)):
        if not np.all(np.isfinite(v)):
            raise ValueError("request %s: %s holds NaN or Inf" % (req.id, name))
    if req.fit not in ("l2", "kl"):
        raise ValueError("request %s: fit must be 'l2' or 'kl'" % req.id)
    if req.fit == "kl" and not req.background > 0:
        raise ValueError("request %s: the KL fit needs a positive background" % req.id)
    if int(req.max_iter) < 1 or not req.tol >= 0:
        raise ValueError("request %s: max_iter >= 1 and tol >= 0" % req.id)
    if req.reg is not None:
        kind = getattr(req.reg, "kind", None)
        if kind not in engine.REG_KINDS or not hasattr(req.reg, "_p"):
            raise ValueError("request %s: reg must be a device regulariser "
                             "(regularisation.Joubert, Mass, Volume, Radius or Iso)" % req.id)
        p = np.asarray(req.reg._p(), dtype=np.float64)
        if p.size > 8 or not np.all(np.isfinite(p)):
            raise ValueError("request %s: regulariser parameters must be at most 8 finite "
                             "numbers" % req.id)
    if req.data_host is not None:
        d = req.data_host
        shape = (A,) + tuple(v.size for v in det)
        if tuple(d.shape) != shape and d.numel() != int(np.prod(shape)):
            raise ValueError("request %s: data must have shape %s" % (req.id, shape))
        # one summing pass (about 25x cheaper than an elementwise test): a
        # NaN or Inf anywhere makes the sum NaN or Inf; only a finite sum
        # that overflowed needs the elementwise test
        if not math.isfinite(float(d.sum())) and not bool(torch.isfinite(d).all()):
            raise ValueError("request %s: data holds NaN or Inf" % req.id)
    elif req.make_data is None:
        raise ValueError("request %s: no data (data_host or make_data)" % req.id)


_ALIGN = 256
_TORCH_DTYPE = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
                np.dtype(np.int32): torch.int32, np.dtype(np.uint8): torch.uint8}


_DTYPES = {t: np.dtype(t) for t in (np.float32, np.float64, np.int32, np.uint8)}


def _layout(items):
    """Byte layout of (name, dtype, shape) buffers packed at 256-byte
    offsets: ({name: (offset, dtype, shape, nbytes)}, total bytes).  Plain
    integer arithmetic: admission runs this for every request."""
    out, off = {}, 0
    for name, dt, shape in items:
        dt = _DTYPES[dt]
        shape = tuple(int(v) for v in shape)
        k = 1
        for v in shape:
            k *= v
        nb = k * dt.itemsize
        out[name] = (off, dt, shape, nb)
        off += (nb + _ALIGN - 1) // _ALIGN * _ALIGN
    return out, max(off, _ALIGN)


def _typed_views(buf):
    """View maker for a uint8 torch buffer (device or host) whose size is a
    multiple of 8 bytes: the buffer is reinterpreted once per element type,
    and each (offset, dtype, shape) of a _layout becomes one strided view
    of it (admission makes some thirty views per request)."""
    typed = {}

    def view(spec):
        off, dt, shape, _nb = spec
        t = typed.get(dt)
        if t is None:
            t = typed[dt] = buf.view(_TORCH_DTYPE[dt])
        strides, k = [], 1
        for v in reversed(shape):
            strides.append(k)
            k *= v
        return t.as_strided(shape, tuple(reversed(strides)), off // dt.itemsize)
    return view


def _host_view(arr, spec):
    """Typed view of a uint8 numpy array."""
    off, dt, shape, nb = spec
    return arr[off:off + nb].view(dt).reshape(shape)


# Pinned host buffers, pooled by power-of-two capacity for the life of the
# process: pinning memory is a slow driver call, and a request needs two
# buffers (input staging, results).  At most _PINNED_KEEP free buffers are
# kept per capacity; the rest are released.
_pinned_free = {}
_PINNED_KEEP = 64


def _pinned_take(nbytes):
    cap = 1 << max(12, int(nbytes - 1).bit_length())
    free = _pinned_free.get(cap)
    if free:
        return free.pop()
    return torch.empty(cap, dtype=torch.uint8, pin_memory=True)


def _pinned_give(buf):
    free = _pinned_free.setdefault(buf.numel(), [])
    if len(free) < _PINNED_KEEP:
        free.append(buf)


class _Slot:
    """Device state of one admitted request."""

    def __init__(self, req, stream, device, use_graph=True, iters_per_launch=4,
                 device_loop=True, setup_stream=None, plans=(None, None), build_loop=True,
                 skip_empty=True):
        self.req = req
        # launch schedules of this request's shape class (engine.Plan, or
        # None for the process-wide one): projection, derivatives
        self.plan_p, self.plan_d = plans
        self.stream = stream
        self.dev = device
        self.k = iters_per_launch
        # Buffers are built and filled on a setup stream: the compute stream
        # may still hold queued fits of earlier requests.  A request's device
        # state is two allocations: an input arena, filled from one pinned
        # staging buffer by one copy, and a work arena (fit fields,
        # derivatives, workspaces); every buffer is a view of one of them.
        setup = setup_stream if setup_stream is not None else stream
        t_start = time.perf_counter()
        I0, x0, r0 = (np.asarray(v) for v in req.init)
        n = len(I0)
        det_h, rec, kdet = DeviceGeometry.host_records(req.orientations, req.ortho,
                                                       req.detector)
        dim = kdet + 1
        I32 = I0.astype(np.float32).reshape(n)
        x32 = x0.astype(np.float32).reshape(n, dim)
        r32 = r0.astype(np.float32).reshape(n, -1)
        iso = r32.shape[1] == 1
        if iso:
            r32 = r32.reshape(n)
        P = (2 + dim) if iso else (1 + dim + (3 if dim == 2 else 6))
        theta = np.concatenate([I32.reshape(n, 1), x32, r32.reshape(n, -1)], 1).astype(np.float64)
        L = req.max_iter + MAX_BACKTRACK + 8
        lay, n_in = _layout([("frames", np.float32, rec.shape)] +
                            [("det%d" % k, np.float32, d.shape) for k, d in enumerate(det_h)] +
                            [("I", np.float32, I32.shape), ("x", np.float32, x32.shape),
                             ("r", np.float32, r32.shape), ("tI", np.float32, I32.shape),
                             ("tx", np.float32, x32.shape), ("tr", np.float32, r32.shape),
                             ("theta", np.float64, (n, P)), ("theta_t", np.float64, (n, P)),
                             ("lam", np.float64, (n,)), ("loss", np.float64, (2,)),
                             ("hist", np.float64, (L,)), ("acc", np.int32, (L,)),
                             ("counter", np.int32, (1,))])
        self.staging = _pinned_take(n_in)
        host = self.staging.numpy()
        host[:n_in] = 0
        for name, val in (("frames", rec), ("I", I32), ("x", x32), ("r", r32), ("tI", I32),
                          ("tx", x32), ("tr", r32), ("theta", theta), ("theta_t", theta),
                          ("lam", np.full(n, float(req.lam0)))):
            _host_view(host, lay[name])[...] = val
        for k, d in enumerate(det_h):
            _host_view(host, lay["det%d" % k])[...] = d
        t_host = time.perf_counter()
        self.arena_in = torch.empty(n_in, dtype=torch.uint8, device=device)
        with torch.cuda.stream(setup):
            self.arena_in.copy_(self.staging[:n_in], non_blocking=True)
        vin = _typed_views(self.arena_in)
        v = lambda name: vin(lay[name])
        self.geom = DeviceGeometry.bound(rec, kdet, det_h, v("frames"),
                                         [v("det%d" % k) for k in range(kdet)], device)
        self.cur = engine.DeviceAtoms.wrap(v("I"), v("x"), v("r"))
        self.trial = engine.DeviceAtoms.wrap(v("tI"), v("tx"), v("tr"))
        self.dim, self.iso, self.P = dim, iso, P
        self.theta, self.theta_trial, self.lam = v("theta"), v("theta_t"), v("lam")
        loss = v("loss")
        self.loss_cur, self.loss_trial = loss[0], loss[1]
        self.hist, self.hist_acc, self.counter = v("hist"), v("acc"), v("counter")
        shape = self.geom.shape
        kl = req.fit == "kl"
        ws_p = max(256, engine.workspace_bytes(_lib.GR_OP_PROJECT, self.cur, self.geom,
                                               self.plan_p))
        ws_d = max(256, engine.workspace_bytes(_lib.GR_OP_DERIVS_2, self.cur, self.geom,
                                               self.plan_d))
        reg = req.reg is not None
        # 3D forwards skip the (angle, tile) items no atom meets: their loss
        # comes from a record of the data alone, made once per fit, and their
        # fields, which no derivative reads, are left unwritten
        n_items = engine.fit_items(self.geom, self.plan_p) if skip_empty else 0
        wl, n_work = _layout([("data", np.float32, shape), ("alpha", np.float32, shape),
                              ("alpha_t", np.float32, shape)] +
                             ([("beta", np.float32, shape), ("beta_t", np.float32, shape)]
                              if kl else []) +
                             ([("empty", np.float64, (n_items,))] if n_items else []) +
                             [("f", np.float64, (n,)), ("g", np.float64, (n, P)),
                              ("H", np.float64, (n, P, P)), ("step", np.float64, (n,)),
                              ("ws_p", np.uint8, (ws_p,)), ("ws_d", np.uint8, (ws_d,))] +
                             ([("reg_f", np.float64, (n,)), ("reg_g", np.float64, (n, P)),
                               ("reg_sum", np.float64, ())] if reg else []))
        self.arena_work = torch.empty(n_work, dtype=torch.uint8, device=device)
        vwork = _typed_views(self.arena_work)
        w = lambda name: vwork(wl[name])
        self.data = w("data")
        with torch.cuda.stream(setup):
            if req.data_host is not None:
                self.data.copy_(req.data_host.reshape(shape), non_blocking=True)
            else:
                self.data.copy_(req.make_data(self.geom, device, setup))
        self.alpha, self.alpha_t = w("alpha"), w("alpha_t")
        self.beta, self.beta_t = (w("beta"), w("beta_t")) if kl else (None, None)
        self.f, self.g, self.H, self.step = w("f"), w("g"), w("H"), w("step")
        self.ws_p, self.ws_d = w("ws_p"), w("ws_d")
        self.empty = w("empty") if n_items else None
        if reg:
            self.reg_kind = req.reg.kind
            self.reg_params = np.asarray(req.reg._p(), dtype=np.float64)
            self.reg_f, self.reg_g, self.reg_sum = w("reg_f"), w("reg_g"), w("reg_sum")
        # results come back into pinned memory: history, counter, parameters
        # and loss, read after the completion event without a stream sync
        self.res_layout, n_res = _layout([("hist", np.float64, (L,)), ("acc", np.int32, (L,)),
                                          ("counter", np.int32, (1,)),
                                          ("theta", np.float64, (n, P)),
                                          ("loss", np.float64, (1,)),
                                          ("loss0", np.float64, (1,))])
        self.results = _pinned_take(n_res)
        vres = _typed_views(self.results)
        r = lambda name: vres(self.res_layout[name])
        self.h_hist, self.h_acc, self.h_counter = r("hist"), r("acc"), r("counter")
        self.h_theta, self.h_loss, self.h_loss0 = r("theta"), r("loss"), r("loss0")
        t_bufs = time.perf_counter()
        if setup is not stream:
            ready = torch.cuda.Event()
            ready.record(setup)
            stream.wait_event(ready)
            # the arenas' memory is in use on the compute stream from here
            self.arena_in.record_stream(stream)
            self.arena_work.record_stream(stream)
        t_cap = time.perf_counter()
        with torch.cuda.stream(stream):
            self.event = torch.cuda.Event()
            self.graph = None
            self.loop = None
            self.loss0 = None
            if not build_loop:
                # a member of a batch: the batch's loop runs its iterations
                self.phase_seconds = {"host_prep": t_host - t_start, "buffers": t_bufs - t_host,
                                      "streams": t_cap - t_bufs}
                self.iterations_launched = 0
                return
            if use_graph and device_loop:
                # the whole fit as one graph: the iteration repeats on the
                # device until the device-side stop test ends it
                try:
                    self.loop = engine.FitLoop(stream, self.iterate, self.hist, self.hist_acc,
                                               self.counter, req.max_iter, MAX_BACKTRACK,
                                               req.tol, device, pass_loop=True)
                except _lib.EngineError:
                    self.loop = None
            t_loop = time.perf_counter()
            self.phase_seconds = {"host_prep": t_host - t_start, "buffers": t_bufs - t_host,
                                  "streams": t_cap - t_bufs,
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
        return self.arena_in.numel() + self.arena_work.numel()

    def release(self):
        """Return the pinned buffers to the pool (the request is finished:
        its copies completed before its last event)."""
        for b in (self.staging, self.results):
            if b is not None:
                _pinned_give(b)
        self.staging = self.results = None

    def _current_fields(self, device_loop):
        """Where the current atoms' fit fields live.  In the device loop they
        stay in the trial buffers: the derivatives, their only reader, run
        only right after an accepted trial (or on the first iteration, after
        the prologue), when the trial buffers hold exactly the current
        atoms' fields, so an accepted trial's fields need no copy.  The
        iteration replayed from the host recomputes the derivatives every
        time and keeps a separate copy."""
        return (self.alpha_t, self.beta_t) if device_loop else (self.alpha, self.beta)

    def prologue(self):
        """Fit fields and loss of the starting atoms (once per fit); the
        starting loss is also copied out (the fit's initial loss)."""
        r = self.req
        alpha, beta = self._current_fields(self.loop is not None)
        if self.empty is not None:
            engine.fit_empty_loss_into(self.cur, self.geom, self.data, r.fit, r.background,
                                       self.empty, self.ws_p, plan=self.plan_p)
        engine.fit_forward_into(self.cur, self.geom, self.data, r.fit, r.background, None,
                                alpha, beta, self.loss_cur, self.ws_p, plan=self.plan_p,
                                empty_loss=self.empty)
        self._add_reg_value(self.cur, self.loss_cur)
        self.h_loss0.copy_(self.loss_cur.reshape(1), non_blocking=True)

    def iterate(self, loop=None):
        """One damped-Newton iteration.  The current atoms' fields are always
        valid here (from the prologue, an accepted trial, or unchanged after
        a rejected one), so only the trial is projected.  Captured into a
        device loop (``loop``), the derivatives are skipped after a rejected
        trial: the atoms did not move, so g and H still hold their values."""
        r = self.req
        beta_c = 1.0 if r.fit == "l2" else 0.0
        alpha, beta = self._current_fields(loop is not None)
        with (loop.unless_rejected() if loop is not None else contextlib.nullcontext()):
            engine.atom_derivs_into(self.cur, self.geom, "field", alpha, beta, beta_c,
                                    2, self.f, self.g, self.H, self.ws_d, plan=self.plan_d)
            if r.reg is not None:
                engine.regulariser(self.reg_kind, self.reg_params, self.cur, self.f, self.g,
                                   self.H, accumulate=True, order=2)
        engine.newton_solve_into(self.dim, self.iso, self.g, self.H, self.lam, self.theta,
                                 self.theta_trial, self.step, self.trial, self.dev)
        engine.fit_forward_into(self.trial, self.geom, self.data, r.fit, r.background, None,
                                self.alpha_t, self.beta_t, self.loss_trial, self.ws_p,
                                plan=self.plan_p, empty_loss=self.empty)
        self._add_reg_value(self.trial, self.loss_trial)
        engine.newton_accept_into(self.dim, self.iso, self.loss_cur, self.loss_trial,
                                  self.theta, self.theta_trial, self.lam, 1e-4, r.lam_max,
                                  self.cur, self.trial, self.hist, self.hist_acc,
                                  self.counter, self.dev,
                                  fields=None if loop is not None else
                                  (self.alpha_t, self.alpha, self.beta_t, self.beta))

    def _add_reg_value(self, atoms, loss):
        """With a regulariser, add its value at ``atoms`` to ``loss`` (FP64, on
        the stream: no allocation, so it can be captured)."""
        if self.req.reg is None:
            return
        engine.regulariser(self.reg_kind, self.reg_params, atoms, f=self.reg_f, g=self.reg_g,
                           H=None, accumulate=False, order=1)
        torch.sum(self.reg_f, dim=0, out=self.reg_sum)
        loss.add_(self.reg_sum)

    def _copy_results(self):
        self.h_counter.copy_(self.counter, non_blocking=True)
        self.h_hist.copy_(self.hist, non_blocking=True)
        self.h_acc.copy_(self.hist_acc, non_blocking=True)
        self.h_theta.copy_(self.theta, non_blocking=True)
        self.h_loss.copy_(self.loss_cur.reshape(1), non_blocking=True)

    def _copy_back(self):
        self._copy_results()
        self.event.record(self.stream)

    @property
    def reqs(self):
        return [self.req]

    def result_map(self):
        return {self.req.id: self.result()}

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
        """Parameters, loss and iteration count from the pinned copies (call
        after the completion event: no stream sync, so other requests
        queued on the same stream are not waited for)."""
        c = min(int(self.h_counter[0]), self.req.max_iter)
        acc = self.h_acc.numpy()[:min(c, self.h_acc.numel())]
        accepted = int((acc != 0).sum())
        return {"theta": self.h_theta.numpy().copy(), "loss": float(self.h_loss[0]),
                "loss0": float(self.h_loss0[0]), "iterations": c,
                "rejected": int((acc == 0).sum()), "accepted": accepted,
                # a fit that accepted no step returns its starting atoms
                "status": "ok" if accepted > 0 else "no_progress"}


def batchable(req):
    """Whether a request can run in a batch of small 2D fits (a shared
    engine.BatchLoop): 2D, L2, no regulariser, at most 224 atoms and 8192
    (angle, 32-cell tile) items.  The engine checks the rest."""
    if len(req.detector) != 1 or req.fit != "l2" or req.reg is not None:
        return False
    n = len(req.init[0])
    tiles = -(-len(np.asarray(req.detector[0]).reshape(-1)) // 32)
    return 1 <= n <= 224 and len(req.orientations) * tiles <= 8192


def _r_layout(req):
    return np.asarray(req.init[2]).reshape(len(req.init[0]), -1).shape[1]


class _BatchSlot:
    """Small 2D fits admitted together: each keeps its own buffers (a _Slot
    built without a loop of its own) and one engine.BatchLoop runs all their
    iterations, every kernel of an iteration one launch over the batch.  A
    request's result is the one its own device loop gives (the batch runs
    the same block bodies on the same buffers)."""

    def __init__(self, reqs, stream, device, setup_stream):
        t0 = time.perf_counter()
        self.stream = stream
        self.members = [_Slot(r, stream, device, True, 1, True, setup_stream, (None, None),
                              build_loop=False) for r in reqs]
        t1 = time.perf_counter()
        self.loop = engine.BatchLoop(self.members, stream, setup_stream, device, MAX_BACKTRACK)
        self.phase_seconds = {}
        for m in self.members:
            for k, v in m.phase_seconds.items():
                self.phase_seconds[k] = self.phase_seconds.get(k, 0.0) + v
        self.phase_seconds["batch_loop"] = time.perf_counter() - t1
        self.phase_seconds["batch_members"] = t1 - t0
        with torch.cuda.stream(stream):
            self.event = torch.cuda.Event()
        self.req = reqs[0]

    @property
    def reqs(self):
        return [m.req for m in self.members]

    def launch(self):
        with torch.cuda.stream(self.stream):
            self.loop.prologue()
            for m in self.members:
                m.h_loss0.copy_(m.loss_cur.reshape(1), non_blocking=True)
            self.loop.launch_loop()
            for m in self.members:
                m._copy_results()
            self.event.record(self.stream)

    def done(self):
        return True

    def result_map(self):
        return {m.req.id: m.result() for m in self.members}

    def release(self):
        for m in self.members:
            m.release()


_warmed = set()


def _work_size(req):
    return req.size_hint[0] * req.size_hint[1]


def promote_when_idle(pending, now, n_active, n_streams):
    """Admission order under ``largest_first="when_idle"``: while fewer than
    half the streams hold a fit (a server starting on a full queue), the
    largest request that has arrived moves to the head of ``pending`` (a
    deque in arrival order; ties keep the earlier one), so the device gets
    long work while the host sets up the next requests.  Otherwise the order
    is left alone.  Returns the promoted request or None."""
    if n_active >= n_streams // 2:
        return None
    best = None
    for i, r in enumerate(pending):
        if r.arrival <= now and (best is None or _work_size(r) > _work_size(best[1])):
            best = (i, r)
    if best is None:
        return None
    if best[0] > 0:
        del pending[best[0]]
        pending.appendleft(best[1])
    return best[1]


def _warm_engine(device):
    """Run every kernel family once eagerly on tiny 2D and 3D problems, so
    that the library's one-time per-device set-up happens outside any stream
    capture."""
    if device in _warmed:
        return
    engine.preload(device)
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
                 largest_first="when_idle", exclusive_streams=True, tuned=False, batch_max=1,
                 skip_empty=True):
        self.dev = torch.device(device or "cuda")
        self.skip_empty = skip_empty
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
        self.exclusive_streams = exclusive_streams
        self.pending = collections.deque()
        self.active = []
        self.results = {}
        self.in_use = 0
        self.stream_busy = [0] * n_streams
        self.admitted_while_busy = 0
        self.admit_seconds = 0.0     # host time spent setting up admitted requests
        self.admit_phases = {}       # the same by phase (buffers, streams, capture)
        self.device_loops = 0        # requests run as one device-resident loop graph
        # Finished requests' loop graphs are destroyed only when no fit runs
        # and more requests are waiting to arrive (an idle moment of a
        # running server), or by close(): destroying an executable graph
        # waits for the whole device to idle, which would stall the host loop
        # behind every fit in flight, and the last results should not wait
        # for the clean-up of all the others.
        self._retired_loops = []
        # launches of each request run under the plans tuned for its shape
        # class (tune_classes), when there are any
        self.tuned = tuned
        self._hold_admission = False
        self.admission_retries = 0   # admissions that failed and were retried
        self.cancelled = set()       # ids of requests cancelled while in flight
        self.errors = {}             # id -> reason, for requests that could not run
        self._admit_fault = None     # test hook: called before a slot is built
        # small 2D fits admitted together share one batched device loop (up
        # to batch_max per batch; 1: every fit runs its own loop)
        self.batch_max = batch_max if (device_loop and use_graphs) else 1
        self.batches = 0
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
        """Queue a request.  Malformed requests are refused here
        (ValueError, see validate_request) and never reach the device."""
        validate_request(req)
        self.pending.append(req)

    def cancel(self, rid):
        """Cancel a request.  A queued one leaves the queue; one in flight
        runs to the end of its device work (nothing is killed on the
        device), after which its result is discarded and its memory freed.
        The request's result is then {"status": "cancelled"}.  Returns
        False if the request is unknown or already finished."""
        for req in list(self.pending):
            if req.id == rid:
                self.pending.remove(req)
                self.results[rid] = {"status": "cancelled", "arrival": req.arrival}
                return True
        if any(r.id == rid for slot in self.active for r in slot.reqs):
            self.cancelled.add(rid)
            return True
        return False

    def _plans(self, req):
        if not self.tuned:
            return None, None
        from . import tuning
        return tuning.plans_for_request(req)

    def _admit(self, now):
        if self._hold_admission:
            return                      # retry only after a fit has finished
        if self.largest_first and self.largest_first != "when_idle" and len(self.pending) > 1:
            # among the requests that have arrived, the largest go first, so
            # the longest fits start early (arrival order otherwise kept);
            # "both ends": largest and smallest alternately, so the small
            # fits, whose time is mostly their host set-up and launch
            # latency, run beside the large ones instead of after them
            arrived = [r for r in self.pending if r.arrival <= now]
            if len(arrived) > 1:
                later = [r for r in self.pending if r.arrival > now]
                arrived.sort(key=lambda r: -(r.size_hint[0] * r.size_hint[1]))
                if self.largest_first == "both_ends":
                    lo, hi, mixed = 0, len(arrived) - 1, []
                    while lo <= hi:
                        mixed.append(arrived[lo])
                        if hi > lo:
                            mixed.append(arrived[hi])
                        lo, hi = lo + 1, hi - 1
                    arrived = mixed
                self.pending = collections.deque(arrived + later)
        while self.pending and len(self.active) < self.max_slots:
            if self.largest_first == "when_idle":
                promote_when_idle(self.pending, now, len(self.active), len(self.streams))
            req = self.pending[0]
            if req.arrival > now:
                break
            si = int(np.argmin(self.stream_busy))
            if self.exclusive_streams and self.stream_busy[si] > 0:
                break                            # wait for a stream of its own
            need = self.estimate_bytes(req)
            if self.in_use + need > self.budget:
                if not self.active:
                    raise MemoryError("request %s needs %d bytes, budget %d"
                                      % (req.id, need, self.budget))
                break
            self.pending.popleft()
            group = [req]
            if self.batch_max > 1 and batchable(req):
                # the other arrived requests that can share its batch, in
                # queue order, as long as the budget holds
                for r in list(self.pending):
                    if len(group) >= self.batch_max or r.arrival > now:
                        break
                    if batchable(r) and _r_layout(r) == _r_layout(req):
                        nr = self.estimate_bytes(r)
                        if self.in_use + need + nr > self.budget:
                            break
                        group.append(r)
                        need += nr
                for r in group[1:]:
                    self.pending.remove(r)
            ta = time.perf_counter()
            try:
                if self._admit_fault is not None:
                    self._admit_fault(req)
                if len(group) > 1 or (self.batch_max > 1 and batchable(req)):
                    slot = _BatchSlot(group, self.streams[si], self.dev, self.setup_stream)
                    self.batches += 1
                else:
                    slot = _Slot(req, self.streams[si], self.dev, self.use_graphs, self.k,
                                 self.device_loop, self.setup_stream, self._plans(req),
                                 skip_empty=self.skip_empty)
            except _lib.EngineError as e:
                self.admit_seconds += time.perf_counter() - ta
                if len(group) > 1:
                    # the batch could not be built: its requests go back to
                    # the head of the queue and run one fit per loop
                    for r in reversed(group):
                        self.pending.appendleft(r)
                    self.batch_max = 1
                    continue
                # the engine refused the request's set-up: it cannot run
                self.errors[req.id] = "%s: %s" % (type(e).__name__, e)
                self.results[req.id] = {"status": "error", "error": self.errors[req.id],
                                        "arrival": req.arrival}
                continue
            except torch.cuda.OutOfMemoryError as e:
                # the device could not take the request now: whatever the
                # slot had allocated is garbage once this frame ends.  With
                # fits in flight it waits (at the head of the queue) until
                # one finishes; with none it can never fit.
                self.admit_seconds += time.perf_counter() - ta
                if not self.active and len(group) == 1:
                    self.errors[req.id] = "%s: %s" % (type(e).__name__, e)
                    self.results[req.id] = {"status": "error", "error": self.errors[req.id],
                                            "arrival": req.arrival}
                    continue
                for r in reversed(group):
                    self.pending.appendleft(r)
                if not self.active:
                    self.batch_max = 1       # alone the fits may still fit
                    continue
                self.admission_retries += 1
                self._hold_admission = True
                break
            self.stream_busy[si] += 1
            if self.active:
                self.admitted_while_busy += 1
            self.admit_seconds += time.perf_counter() - ta
            phases = dict(slot.phase_seconds)
            if slot.loop is not None and hasattr(slot.loop, "seconds"):
                phases.update(slot.loop.seconds)
            for k, v in phases.items():
                self.admit_phases[k] = self.admit_phases.get(k, 0.0) + v
            slot.stream_index = si
            if slot.loop is not None:
                self.device_loops += len(slot.reqs)
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
                if slot.done() or any(r.id in self.cancelled for r in slot.reqs):
                    fin = time.perf_counter() - t0
                    done_reqs = []
                    all_res = slot.result_map()
                    for r in slot.reqs:
                        res = all_res[r.id]
                        if r.id in self.cancelled:
                            self.cancelled.discard(r.id)
                            res = {"status": "cancelled"}
                        res["arrival"] = r.arrival
                        res["admitted"] = slot.t_admit - t0
                        res["finish"] = fin
                        res["latency"] = fin - r.arrival
                        self.results[r.id] = res
                        done_reqs.append((r, res))
                    self.active.remove(slot)
                    self._hold_admission = False
                    self.in_use -= slot.need
                    self.stream_busy[slot.stream_index] -= 1
                    if slot.loop is not None:
                        self._retired_loops.append(slot.loop)
                        slot.loop = None
                    slot.release()
                    if on_done:
                        for r, res in done_reqs:
                            on_done(r, res)
                    del slot
                    if not self.active and self.pending:
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
        return self.results

    def close(self):
        """Destroy the loop graphs of the finished fits (waits for the device
        to idle); the server can take more requests afterwards."""
        self._release_loops()

    def _release_loops(self):
        """Destroy the retired loop graphs (nothing of this server runs)."""
        if self._retired_loops:
            torch.cuda.synchronize(self.dev)
            for lp in self._retired_loops:
                lp.close()
            self._retired_loops = []


def serve_plain(requests, device=None, t0=None, lean=False):
    """Baseline: the same fits one at a time with the eager host-driven loop
    (no graphs, no overlap); a request starts at max(arrival, previous end).
    lean=False keeps the reference loop's structure (NewtonGaussian.py:57-60
    evaluates the derivatives on every inner iteration, and the current
    atoms are projected anew each iteration); lean=True does only the work
    the served loop does (one projection per iteration, no derivatives after
    a rejected trial).  Both give the same fits."""
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
        cur, losses, accepted, trials = _plain_fit(atoms, geom, data, req, lean)
        torch.cuda.synchronize(dev)
        fin = time.perf_counter() - t0
        # iterations: trials, accepted or not (as the served loop counts them)
        out[req.id] = {"loss": losses[-1], "loss0": losses[0], "iterations": trials,
                       "accepted": accepted, "status": "ok" if accepted else "no_progress",
                       "arrival": req.arrival, "finish": fin, "latency": fin - req.arrival}
    return out


def _plain_fit(atoms, geom, data, req, lean=False):
    """Eager damped Newton with the same accept rule and stopping test.
    Returns (atoms, loss after every accepted step, accepted steps, trials)."""
    from . import solvers
    dim, iso = atoms.dim, atoms.iso
    theta = solvers.theta_of(atoms.I, atoms.x, atoms.r)
    fit, bg = req.fit, req.background
    beta_c = 1.0 if fit == "l2" else 0.0
    lam = torch.full((atoms.n,), float(req.lam0), dtype=torch.float64, device=geom.device)
    cur = atoms
    losses = []
    rejects = 0
    accepted = 0
    reg = req.reg
    # with a regulariser: its value joins the loss, its terms the blocks
    reg_value = (lambda a: float(reg.terms(a, order=1)[0].sum().item())) if reg else (lambda a: 0.0)
    fw = engine.fit_forward(cur, geom, data, fit, bg)
    loss = float(fw["loss"].item()) + reg_value(cur)
    g = H = None
    trials = 0
    for it in range(req.max_iter):
        trials += 1
        if not lean and it > 0:
            fw = engine.fit_forward(cur, geom, data, fit, bg)
            loss = float(fw["loss"].item()) + reg_value(cur)
        if not losses:
            losses.append(loss)
        if g is None or not lean or rejects == 0:
            f_, g, H = engine.atom_derivs(cur, geom, "field", fw["alpha"], fw["beta"], beta_c, 2)
            if reg:
                reg.device_terms(cur, f_, g, H)
        th, _s, _fl = engine.newton_solve(dim, iso, g.contiguous(), H.contiguous(), lam, theta)
        trial = solvers.atoms_of(th, dim, geom.device)
        fwt = engine.fit_forward(trial, geom, data, fit, bg, want_fields=lean)
        new = float(fwt["loss"].item()) + reg_value(trial)
        if new <= loss:
            theta, cur = th, trial
            if lean:
                fw = fwt
            lam = torch.clamp(lam / 2, 1e-4, req.lam_max)
            losses.append(new)
            rejects = 0
            accepted += 1
            prev, loss = loss, new
            if abs(prev - new) <= req.tol * max(abs(prev), 1e-300):
                break
        else:
            lam = torch.clamp(lam * 10, 1e-4, req.lam_max)
            rejects += 1
            if rejects >= MAX_BACKTRACK:
                break
    return cur, losses, accepted, trials
