"""Device-level API of the Gaussian-atom Radon engine (torch tensors in HBM).

Every function here launches the hand-written sm_103a kernels of
libgauss_radon.so through its C ABI on the current torch CUDA stream.  There
is no CPU path: calls raise ``EngineError`` when the library or a CUDA device
is missing.

Atoms are ``(I (N,), x (N, d), r (N, P_r) or (N,) / (N, 1) isotropic)``;
geometry is a :class:`DeviceGeometry`.
"""
import contextlib
import ctypes
import threading

import numpy as np
import torch

from . import _lib
from .geometry import DeviceGeometry

_ws_lock = threading.Lock()
_workspaces = {}


def _require_cuda(device):
    if not torch.cuda.is_available():
        raise _lib.EngineError("no CUDA device: the Gaussian-atom Radon engine "
                               "runs only on the GPU")
    if device.type != "cuda":
        raise _lib.EngineError("engine tensors must live on a CUDA device, got %s" % device)


def workspace(nbytes, device):
    """Per-(device, stream) scratch buffer, grown on demand and reused."""
    stream = torch.cuda.current_stream(device)
    key = (device.index, stream.cuda_stream)
    with _ws_lock:
        buf = _workspaces.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
            _workspaces[key] = buf
    return buf


def _stream_handle(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def morton_order(x):
    """Permutation visiting atom centres x (N, d) along a Morton (Z-order)
    curve of a 2^10-per-axis grid over their bounding box, so consecutive
    atoms are spatially close."""
    import numpy as np
    x = np.asarray(x, dtype=np.float64)
    n, d = x.shape
    lo, hi = x.min(axis=0), x.max(axis=0)
    q = ((x - lo) / np.maximum(hi - lo, 1e-12) * 1023).astype(np.uint64)
    code = np.zeros(n, dtype=np.uint64)
    for bit in range(10):
        for k in range(d):
            code |= ((q[:, k] >> np.uint64(bit)) & np.uint64(1)) << np.uint64(bit * d + k)
    return np.argsort(code, kind="stable").astype(np.int32)


class DeviceAtoms:
    """Float32 device copies of atom parameters plus the C-ABI descriptor.

    order: None (index order), "spatial" (Morton order of the centres, better
    cache locality in the derivative kernels for large atom sets), or a
    permutation; results do not depend on it."""

    def __init__(self, I, x, r, device=None, order=None):
        device = torch.device(device or "cuda")
        _require_cuda(device)
        I = torch.as_tensor(I).to(device=device, dtype=torch.float32).reshape(-1).contiguous()
        n = I.numel()
        x = torch.as_tensor(x).to(device=device, dtype=torch.float32)
        r = torch.as_tensor(r).to(device=device, dtype=torch.float32)
        if n > 0:
            x = x.reshape(n, -1).contiguous()
            r = r.reshape(n, -1).contiguous()
        else:
            x = x.reshape(0, x.shape[-1] if x.dim() > 1 else 0)
            r = r.reshape(0, r.shape[-1] if r.dim() > 1 else 1)
        if r.shape[1] == 1:
            r = r.reshape(n).contiguous()
        self._bind(I, x, r, device, order)

    @classmethod
    def wrap(cls, I, x, r):
        """Atoms over float32 device tensors I (n,), x (n, dim) and r (n,)
        (isotropic) or (n, 3 | 6), used in place: no allocation, no copy."""
        self = cls.__new__(cls)
        self._bind(I, x, r, I.device, None)
        return self

    def _bind(self, I, x, r, device, order):
        n = I.numel()
        self.iso = r.dim() == 1
        self.I, self.x, self.r = I, x, r
        self.n = n
        self.dim = x.shape[1] if n > 0 else 0
        s = _lib.GrAtoms()
        s.n_atoms = n
        s.I = I.data_ptr() if n else None
        s.x = x.data_ptr() if n else None
        s.r = r.data_ptr() if n else None
        s.r_iso = 1 if self.iso else 0
        self.order = None
        if isinstance(order, str) and order == "spatial" and n > 1:
            order = morton_order(x.detach().cpu().numpy())
        if order is not None and not isinstance(order, str):
            self.order = torch.as_tensor(order, dtype=torch.int32).to(device).contiguous()
            if self.order.numel() != n:
                raise ValueError("order must be a permutation of the atoms")
        s.order = self.order.data_ptr() if self.order is not None else None
        self.struct = s

    def n_params(self):
        d = self.dim
        if self.iso:
            return 2 + d
        return 1 + d + (3 if d == 2 else 6)


def _check_dims(atoms, geom):
    if atoms.n and atoms.dim != geom.dim:
        raise ValueError("atoms are %dD but the geometry is %dD" % (atoms.dim, geom.dim))
    if not atoms.iso and atoms.n:
        want = 3 if geom.dim == 2 else 6
        if atoms.r.shape[1] != want:
            raise ValueError("anisotropic r must have %d entries per atom" % want)


class Plan:
    """A launch schedule (work split and tiling) owned by the caller: the
    C ABI's gr_plan.  Engine calls given ``plan=`` run under it instead of
    the process-wide values of gr_set_tuning, so fits on concurrent streams
    can each use the schedule tuned for their shape class.  Created from the
    current process-wide values; ``set``/``get`` take the GR_TUNE_* keys."""

    def __init__(self, op, atoms, geom):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.gr_plan_create(int(op), ctypes.byref(atoms.struct),
                                      ctypes.byref(geom.struct), ctypes.byref(h)),
                   "gr_plan_create")
        self._h = h
        self.op = int(op)

    @property
    def handle(self):
        return self._h

    def set(self, key, value):
        _lib.check(_lib.load().gr_plan_set(self._h, int(key), int(value)), "gr_plan_set")
        return self

    def get(self, key):
        return int(_lib.load().gr_plan_get(self._h, int(key)))

    def workspace_bytes(self, op, atoms, geom):
        return int(_lib.load().gr_plan_workspace_bytes(self._h, int(op),
                                                       ctypes.byref(atoms.struct),
                                                       ctypes.byref(geom.struct)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().gr_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ws_for(op, atoms, geom, plan=None):
    if plan is not None:
        n = plan.workspace_bytes(op, atoms, geom)
    else:
        n = _lib.load().gr_workspace_bytes(op, ctypes.byref(atoms.struct),
                                           ctypes.byref(geom.struct))
    return workspace(n, geom.device), n


def _fn(name, psf, plan):
    """The entry point for a call: psf variant, or the plan-taking variant
    (bound to the plan's handle)."""
    lib = _lib.load()
    if plan is None:
        return getattr(lib, ("gr_psf_" + name) if psf else ("gr_" + name))
    if psf:
        raise ValueError("plans cover the point-sampled operator")
    f = getattr(lib, "gr_%s_plan" % name)
    return lambda *a: f(plan.handle, *a)


def radproj(atoms, geom, out=None, psf=False, plan=None):
    """Forward projection R (A, D0[, D1]) float32 on the device; psf=True
    gives the pixel-integrated (single-particle) projection."""
    _check_dims(atoms, geom)
    if out is None:
        out = torch.empty(geom.shape, dtype=torch.float32, device=geom.device)
    if tuple(out.shape) != tuple(geom.shape) or out.dtype != torch.float32 or not out.is_contiguous():
        raise ValueError("output must be a contiguous float32 tensor of shape %s" % (geom.shape,))
    ws, n = _ws_for(_lib.GR_OP_PROJECT, atoms, geom, plan)
    fn = _fn("radproj", psf, plan)
    st = fn(ctypes.byref(atoms.struct), ctypes.byref(geom.struct),
            out.data_ptr(), ws.data_ptr(), n, _stream_handle(geom.device))
    _lib.check(st, "gr_radproj")
    return out


def fit_forward(atoms, geom, data, fit="l2", background=0.0, want_R=False,
                want_fields=True, psf=False, plan=None):
    """Projection fused with an L2 or KL fit.

    Returns dict with 'loss' (0-d float64 device tensor), 'alpha', 'beta'
    (KL) and 'R' when requested.
    """
    _check_dims(atoms, geom)
    data = torch.as_tensor(data, device=geom.device, dtype=torch.float32).contiguous()
    if tuple(data.shape) != tuple(geom.shape):
        raise ValueError("data shape %s does not match geometry %s" % (tuple(data.shape), geom.shape))
    code = {"l2": _lib.GR_FIT_L2, "kl": _lib.GR_FIT_KL}[fit]
    dev = geom.device
    out = {"loss": torch.empty((), dtype=torch.float64, device=dev)}
    R = torch.empty(geom.shape, dtype=torch.float32, device=dev) if want_R else None
    alpha = torch.empty(geom.shape, dtype=torch.float32, device=dev) if want_fields else None
    beta = (torch.empty(geom.shape, dtype=torch.float32, device=dev)
            if (want_fields and fit == "kl") else None)
    ws, n = _ws_for(_lib.GR_OP_PROJECT, atoms, geom, plan)
    p = lambda t: None if t is None else t.data_ptr()
    fn = _fn("fit_forward", psf, plan)
    st = fn(
        ctypes.byref(atoms.struct), ctypes.byref(geom.struct), code, data.data_ptr(),
        float(background), p(R), p(alpha), p(beta), out["loss"].data_ptr(),
        ws.data_ptr(), n, _stream_handle(dev))
    _lib.check(st, "gr_fit_forward")
    out["R"], out["alpha"], out["beta"] = R, alpha, beta
    return out


MODES = {"field": _lib.GR_MODE_FIELD, "l2_atom": _lib.GR_MODE_L2_ATOM,
         "inner": _lib.GR_MODE_INNER}


def atom_derivs(atoms, geom, mode, field, beta_field=None, beta_const=1.0, order=2,
                psf=False, plan=None):
    """Per-atom value (N,), gradient (N, P) and Hessian (N, P, P), float64.

    mode 'inner' (field = C): derivatives of <R_j, C>;
    mode 'l2_atom' (field = C): of 1/2 |R_j - C|^2, each atom alone;
    mode 'field' (field = alpha, beta): g = sum alpha dR_j,
    H = sum beta dR_j dR_j^T + alpha d2R_j, f = 0.
    """
    _check_dims(atoms, geom)
    dev = geom.device
    field = torch.as_tensor(field, device=dev, dtype=torch.float32).contiguous()
    if tuple(field.shape) != tuple(geom.shape):
        raise ValueError("field shape %s does not match geometry %s" % (tuple(field.shape), geom.shape))
    if beta_field is not None:
        beta_field = torch.as_tensor(beta_field, device=dev, dtype=torch.float32).contiguous()
    P = atoms.n_params()
    N = atoms.n
    f = torch.empty(N, dtype=torch.float64, device=dev)
    g = torch.empty((N, P), dtype=torch.float64, device=dev)
    H = torch.empty((N, P, P), dtype=torch.float64, device=dev) if order == 2 else None
    if N == 0:
        return f, g, H
    op = _lib.GR_OP_DERIVS_1 if order == 1 else _lib.GR_OP_DERIVS_2
    ws, n = _ws_for(op, atoms, geom, plan)
    fn = _fn("atom_derivs", psf, plan)
    st = fn(
        ctypes.byref(atoms.struct), ctypes.byref(geom.struct), MODES[mode],
        field.data_ptr(), None if beta_field is None else beta_field.data_ptr(),
        float(beta_const), int(order), f.data_ptr(), g.data_ptr(),
        None if H is None else H.data_ptr(), ws.data_ptr(), n, _stream_handle(dev))
    _lib.check(st, "gr_atom_derivs")
    return f, g, H


def l2_fit_derivs(atoms, geom, data, order=2):
    """Loss 1/2|R - data|^2 and, for every atom j, the gradient and Hessian of
    the reference's L2derivs_RadProj(atom_j, data + R_j - R) (the Newton-loop
    call, NewtonGaussian.py:59-60).  f_j equals the loss for every j."""
    fw = fit_forward(atoms, geom, data, "l2")
    f, g, H = atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, order)
    f.copy_(fw["loss"].expand_as(f))
    return fw["loss"], g, H


def kl_fit_derivs(atoms, geom, data, background, order=2):
    """KL(data || R + b) with its per-atom gradient and Hessian."""
    fw = fit_forward(atoms, geom, data, "kl", background)
    f, g, H = atom_derivs(atoms, geom, "field", fw["alpha"], fw["beta"], 0.0, order)
    f.copy_(fw["loss"].expand_as(f))
    return fw["loss"], g, H


def count_support(atoms, geom):
    """Exact number of (atom, angle, cell) triples with m <= 1 (int)."""
    _check_dims(atoms, geom)
    out = torch.zeros(1, dtype=torch.int64, device=geom.device)
    st = _lib.load().gr_count_support(ctypes.byref(atoms.struct), ctypes.byref(geom.struct),
                                      out.data_ptr(), _stream_handle(geom.device))
    _lib.check(st, "gr_count_support")
    return int(out.item())


def probe_ex2(blocks, threads, iters, device=None):
    """Launch the ex2 throughput probe (blocks*threads*iters*8 operations)."""
    device = torch.device(device or "cuda")
    _require_cuda(device)
    sink = torch.zeros(1, dtype=torch.float32, device=device)
    st = _lib.load().gr_probe_ex2(int(blocks), int(threads), int(iters), sink.data_ptr(),
                                  _stream_handle(device))
    _lib.check(st, "gr_probe_ex2")


TIMER_PROJECT, TIMER_DERIVS = 1, 2


def kernel_timer(which, enable=True):
    """Start (clearing) or stop the CUDA-event timer around the projection
    (TIMER_PROJECT) or derivative (TIMER_DERIVS) kernel launches."""
    _lib.check(_lib.load().gr_kernel_timer(int(which), 1 if enable else 0), "gr_kernel_timer")


def kernel_timer_read(which):
    """(summed ms, launches) of the timed kernel launches (waits for them)."""
    ms, n = ctypes.c_double(), ctypes.c_int()
    _lib.check(_lib.load().gr_kernel_timer_read(int(which), ctypes.byref(ms), ctypes.byref(n)),
               "gr_kernel_timer_read")
    return ms.value, n.value


def launch_count():
    """Kernels launched by the engine library so far in this process."""
    return int(_lib.load().gr_launch_count())


def atom_step(old_atom, new_atom, geom, fit, apply, R, data, alpha, beta=None,
              background=0.0, dloss=None):
    """Trial (apply=False: returns the fit change as a 0-d float64 device
    tensor) or application (apply=True) of one atom's move; see
    gr_atom_step in include/gauss_radon.h."""
    code = {"l2": _lib.GR_FIT_L2, "kl": _lib.GR_FIT_KL}[fit]
    dev = geom.device
    if dloss is None and not apply:
        dloss = torch.empty((), dtype=torch.float64, device=dev)
    ws, n = _ws_for(_lib.GR_OP_ATOM_STEP, old_atom, geom)
    p = lambda t: None if t is None else t.data_ptr()
    st = _lib.load().gr_atom_step(
        ctypes.byref(old_atom.struct), ctypes.byref(new_atom.struct), ctypes.byref(geom.struct),
        code, 1 if apply else 0, R.data_ptr(), data.data_ptr(), float(background),
        alpha.data_ptr(), p(beta), p(dloss), ws.data_ptr(), n, _stream_handle(dev))
    _lib.check(st, "gr_atom_step")
    return dloss


def newton_solve(dim, iso, g, H, lam, theta, mask=None):
    """Batched damped Newton update (FP64) with the reference's clamps.
    Returns (theta_new (N, P), step_norm (N,), fail (N,) int32)."""
    n = theta.shape[0]
    dev = theta.device
    theta_new = torch.empty_like(theta)
    step = torch.empty(n, dtype=torch.float64, device=dev)
    fail = torch.empty(n, dtype=torch.int32, device=dev)
    for t in (g, H, lam, theta):
        assert t.dtype == torch.float64 and t.is_contiguous()
    st = _lib.load().gr_newton_solve(
        int(dim), 1 if iso else 0, int(n), g.data_ptr(), H.data_ptr(), lam.data_ptr(),
        theta.data_ptr(), None if mask is None else mask.data_ptr(), theta_new.data_ptr(),
        step.data_ptr(), fail.data_ptr(), None, None, None, _stream_handle(dev))
    _lib.check(st, "gr_newton_solve")
    return theta_new, step, fail


# ---------------------------------------------------------------------------
# allocation-free forms with caller-owned buffers (CUDA-graph capturable)
# ---------------------------------------------------------------------------
def preload(device=None):
    """Load every kernel of the library on ``device`` now (see gr_preload)."""
    device = torch.device(device or "cuda")
    _require_cuda(device)
    with torch.cuda.device(device):
        _lib.check(_lib.load().gr_preload(), "gr_preload")


def workspace_bytes(op, atoms, geom, plan=None):
    if plan is not None:
        return plan.workspace_bytes(op, atoms, geom)
    return int(_lib.load().gr_workspace_bytes(op, ctypes.byref(atoms.struct),
                                              ctypes.byref(geom.struct)))


def _ptr(t):
    return None if t is None else t.data_ptr()


def fit_items(geom, plan=None):
    """(angle, tile) items of the 3D forward that can skip the items no atom
    meets (0 for 2D geometries, which do not skip)."""
    n = ctypes.c_size_t(0)
    _lib.check(_lib.load().gr_fit_items(plan.handle if plan is not None else None,
                                        ctypes.byref(geom.struct), ctypes.byref(n)),
               "gr_fit_items")
    return int(n.value)


def fit_empty_loss_into(atoms, geom, data, fit, background, empty_loss, ws, plan=None):
    """Each item's loss with no atom in it (float64, fit_items(geom, plan)
    entries), under the schedule a forward of ``atoms`` takes: the record
    that fit_forward_into(empty_loss=...) gives the items no atom meets."""
    code = {"l2": _lib.GR_FIT_L2, "kl": _lib.GR_FIT_KL}[fit]
    st = _lib.load().gr_fit_empty_loss(
        plan.handle if plan is not None else None, ctypes.byref(atoms.struct),
        ctypes.byref(geom.struct), code, data.data_ptr(), float(background),
        empty_loss.data_ptr(), empty_loss.numel(), ws.data_ptr(), ws.numel(),
        _stream_handle(geom.device))
    _lib.check(st, "gr_fit_empty_loss")


def fit_forward_into(atoms, geom, data, fit, background, R, alpha, beta, loss, ws, psf=False,
                     plan=None, empty_loss=None):
    """Fused forward into caller buffers.  With ``empty_loss`` (from
    fit_empty_loss_into; 3D, R None) the items no atom meets take their loss
    from it and keep their old field values: the loss is bitwise the same and
    so are the fields wherever an atom is, which is all a Newton iteration's
    derivatives read."""
    code = {"l2": _lib.GR_FIT_L2, "kl": _lib.GR_FIT_KL}[fit]
    if empty_loss is not None:
        if psf or R is not None:
            raise ValueError("skipping empty items needs the point-sampled forward without R")
        st = _lib.load().gr_fit_forward_skip(
            plan.handle if plan is not None else None, ctypes.byref(atoms.struct),
            ctypes.byref(geom.struct), code, data.data_ptr(), float(background), _ptr(alpha),
            _ptr(beta), _ptr(loss), empty_loss.data_ptr(), empty_loss.numel(), ws.data_ptr(),
            ws.numel(), _stream_handle(geom.device))
        _lib.check(st, "gr_fit_forward_skip")
        return
    fn = _fn("fit_forward", psf, plan)
    st = fn(
        ctypes.byref(atoms.struct), ctypes.byref(geom.struct), code, data.data_ptr(),
        float(background), _ptr(R), _ptr(alpha), _ptr(beta), _ptr(loss), ws.data_ptr(),
        ws.numel(), _stream_handle(geom.device))
    _lib.check(st, "gr_fit_forward")


def atom_derivs_into(atoms, geom, mode, field, beta_field, beta_const, order, f, g, H, ws,
                     psf=False, plan=None):
    fn = _fn("atom_derivs", psf, plan)
    st = fn(
        ctypes.byref(atoms.struct), ctypes.byref(geom.struct), MODES[mode], field.data_ptr(),
        _ptr(beta_field), float(beta_const), int(order), f.data_ptr(), g.data_ptr(), _ptr(H),
        ws.data_ptr(), ws.numel(), _stream_handle(geom.device))
    _lib.check(st, "gr_atom_derivs")


def newton_solve_into(dim, iso, g, H, lam, theta, theta_new, step, trial_atoms, device):
    st = _lib.load().gr_newton_solve(
        int(dim), 1 if iso else 0, int(theta.shape[0]), g.data_ptr(), H.data_ptr(),
        lam.data_ptr(), theta.data_ptr(), None, theta_new.data_ptr(), step.data_ptr(), None,
        trial_atoms.I.data_ptr(), trial_atoms.x.data_ptr(), trial_atoms.r.data_ptr(),
        _stream_handle(device))
    _lib.check(st, "gr_newton_solve")


def accept_fields_into(loss_cur, loss_trial, alpha_t, alpha, beta_t, beta, device):
    """Trial fields become the current ones if the trial was accepted."""
    st = _lib.load().gr_accept_fields(
        loss_cur.data_ptr(), loss_trial.data_ptr(), alpha_t.data_ptr(), alpha.data_ptr(),
        _ptr(beta_t), _ptr(beta), int(alpha.numel()), _stream_handle(device))
    _lib.check(st, "gr_accept_fields")


def newton_accept_into(dim, iso, loss_cur, loss_trial, theta, theta_trial, lam, lam_min,
                       lam_max, cur_atoms, trial_atoms, hist, hist_acc, counter, device,
                       fields=None):
    """Device-side accept/reject; ``fields = (alpha_t, alpha, beta_t, beta)``
    also adopts the trial's fit fields when it is accepted (one launch)."""
    args = (int(dim), 1 if iso else 0, int(theta.shape[0]), loss_cur.data_ptr(),
            loss_trial.data_ptr(), theta.data_ptr(), theta_trial.data_ptr(), lam.data_ptr(),
            float(lam_min), float(lam_max), cur_atoms.I.data_ptr(), cur_atoms.x.data_ptr(),
            cur_atoms.r.data_ptr(), trial_atoms.I.data_ptr(), trial_atoms.x.data_ptr(),
            trial_atoms.r.data_ptr(), hist.data_ptr(), hist_acc.data_ptr(), counter.data_ptr(),
            int(hist.numel()))
    if fields is None:
        st = _lib.load().gr_newton_accept(*args, _stream_handle(device))
        _lib.check(st, "gr_newton_accept")
        return
    alpha_t, alpha, beta_t, beta = fields
    st = _lib.load().gr_newton_accept_fields(
        *args, alpha_t.data_ptr(), alpha.data_ptr(), _ptr(beta_t), _ptr(beta),
        int(alpha.numel()), _stream_handle(device))
    _lib.check(st, "gr_newton_accept_fields")


def _pack(items, align=64):
    """Element offsets of (name, shape) buffers packed at ``align``-element
    boundaries: ({name: (offset, shape)}, total elements)."""
    out, off = {}, 0
    for name, shape in items:
        k = int(np.prod(shape, dtype=np.int64)) if len(shape) else 1
        out[name] = (off, shape)
        off += (k + align - 1) // align * align
    return out, max(off, align)


def _packed_view(buf, spec):
    off, shape = spec
    k = int(np.prod(shape, dtype=np.int64)) if len(shape) else 1
    return buf[off:off + k].view(shape)


class FitStep:
    """One fit evaluation from host inputs to host results, as a CUDA graph.

    Loss, per-atom gradient and (order 2) Hessian of the L2 or KL fit of
    ``n_atoms`` atoms to a sinogram on ``geom``.  The graph holds the
    host->device copies of the atoms and data from this object's pinned host
    buffers, the fused projection + fit (``gr_fit_forward``), the per-atom
    derivatives (``gr_atom_derivs`` in field mode) and the device->host copies
    of loss, gradient and Hessian into pinned host buffers, so one evaluation
    is one graph launch.  ``run`` copies new inputs into the pinned buffers
    (when given), replays and waits; its results are views of the pinned
    output buffers, overwritten by the next run.

    Large sinograms are fitted in ``chunks`` ranges of angles (default: one
    per 128 MB of data, at most 8): a side stream copies range i+1 in while
    the projection of range i runs, so the copy of the data overlaps the
    projection instead of preceding it; the loss is the FP64 sum of the
    ranges' losses, and the derivatives run once over all angles.
    """

    def __init__(self, geom, n_atoms, iso=False, fit="l2", background=0.0, order=2,
                 psf=False, chunks=None):
        dev = geom.device
        _require_cuda(dev)
        if fit not in ("l2", "kl"):
            raise ValueError("fit must be 'l2' or 'kl'")
        self.geom, self.fit, self.order, self.psf = geom, fit, int(order), bool(psf)
        self.background = float(background)
        n, d = int(n_atoms), geom.dim
        pr = 1 if iso else (3 if d == 2 else 6)
        P = (2 + d) if iso else (1 + d + (3 if d == 2 else 6))
        # inputs (atoms, data) and outputs (loss, gradient, Hessian) each live
        # in one arena, on the device and pinned on the host, so a step moves
        # each way with a single copy; every buffer is a view
        ishape = [("I", (n,)), ("x", (n, d)), ("r", (n, pr)), ("data", tuple(geom.shape))]
        oshape = [("loss", ()), ("g", (n, P))] + ([("H", (n, P, P))] if self.order > 1 else [])
        ilay, ni = _pack(ishape)
        olay, no = _pack(oshape)
        self.in_h = torch.zeros(ni, dtype=torch.float32, pin_memory=True)
        self.in_d = torch.zeros(ni, dtype=torch.float32, device=dev)
        self.out_h = torch.zeros(no, dtype=torch.float64, pin_memory=True)
        self.out_d = torch.zeros(no, dtype=torch.float64, device=dev)
        self.I_h, self.x_h, self.r_h, self.data_h = (_packed_view(self.in_h, ilay[k])
                                                     for k, _ in ishape)
        self.I_d, self.x_d, self.r_d, self.data_d = (_packed_view(self.in_d, ilay[k])
                                                     for k, _ in ishape)
        self.r_h.fill_(1.0)
        self.r_d.fill_(1.0)
        self.atoms = DeviceAtoms.wrap(self.I_d, self.x_d, self.r_d.reshape(n) if iso else self.r_d)
        f32 = dict(dtype=torch.float32, device=dev)
        self.alpha = torch.empty(geom.shape, **f32)
        self.beta = torch.empty(geom.shape, **f32) if fit == "kl" else None
        f64 = dict(dtype=torch.float64, device=dev)
        self.f = torch.zeros(n, **f64)
        self.loss = _packed_view(self.out_d, olay["loss"])
        self.g = _packed_view(self.out_d, olay["g"])
        self.H = _packed_view(self.out_d, olay["H"]) if self.order > 1 else None
        self.loss_h = _packed_view(self.out_h, olay["loss"])
        self.g_h = _packed_view(self.out_h, olay["g"])
        self.H_h = _packed_view(self.out_h, olay["H"]) if self.order > 1 else None
        nb = max(workspace_bytes(_lib.GR_OP_PROJECT, self.atoms, geom),
                 workspace_bytes(_lib.GR_OP_DERIVS_2 if self.order > 1 else _lib.GR_OP_DERIVS_1,
                                 self.atoms, geom))
        self.ws = torch.empty(max(nb, 256), dtype=torch.uint8, device=dev)
        # the bytes each step copies (the arenas, with their alignment gaps)
        self.h2d_bytes = self.in_h.numel() * self.in_h.element_size()
        self.d2h_bytes = self.out_h.numel() * self.out_h.element_size()
        A = geom.n_angles
        data_bytes = int(self.data_d.numel()) * 4
        if chunks is None:
            chunks = min(8, (data_bytes + (128 << 20) - 1) >> 27) if data_bytes >= (128 << 20) else 1
        chunks = max(1, min(int(chunks), A))
        bounds = [(i * A) // chunks for i in range(chunks + 1)]
        self.ranges = [(a0, a1, geom.angle_range(a0, a1) if chunks > 1 else geom)
                       for a0, a1 in zip(bounds[:-1], bounds[1:])]
        if chunks > 1:
            self.data_off = ilay["data"][0]
            self.loss_parts = torch.zeros(chunks, **f64)
            self.copy_stream = torch.cuda.Stream(dev)
            self.copied = [torch.cuda.Event() for _ in range(chunks)]
        stream = torch.cuda.Stream(dev)
        stream.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(stream):
            self._body()                     # warm-up outside the capture
        stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=stream):
            self._body()
        torch.cuda.synchronize(dev)

    def _body(self):
        if len(self.ranges) == 1:
            self.in_d.copy_(self.in_h, non_blocking=True)
            fit_forward_into(self.atoms, self.geom, self.data_d, self.fit, self.background, None,
                             self.alpha, self.beta, self.loss, self.ws, psf=self.psf)
        else:
            main = torch.cuda.current_stream(self.geom.device)
            k = self.data_off
            self.in_d[:k].copy_(self.in_h[:k], non_blocking=True)     # the atoms
            self.copy_stream.wait_stream(main)
            with torch.cuda.stream(self.copy_stream):
                for (a0, a1, _g), ev in zip(self.ranges, self.copied):
                    self.data_d[a0:a1].copy_(self.data_h[a0:a1], non_blocking=True)
                    ev.record()
            for i, ((a0, a1, g), ev) in enumerate(zip(self.ranges, self.copied)):
                main.wait_event(ev)
                fit_forward_into(self.atoms, g, self.data_d[a0:a1], self.fit, self.background,
                                 None, self.alpha[a0:a1],
                                 None if self.beta is None else self.beta[a0:a1],
                                 self.loss_parts[i:i + 1], self.ws, psf=self.psf)
            torch.sum(self.loss_parts, dim=0, out=self.loss)
        bc = 1.0 if self.fit == "l2" else 0.0
        atom_derivs_into(self.atoms, self.geom, "field", self.alpha, self.beta, bc, self.order,
                         self.f, self.g, self.H, self.ws, psf=self.psf)
        self.out_h.copy_(self.out_d, non_blocking=True)

    def set_inputs(self, I=None, x=None, r=None, data=None):
        """Copy new atoms and/or data into the pinned input buffers."""
        for src, dst in ((I, self.I_h), (x, self.x_h), (r, self.r_h), (data, self.data_h)):
            if src is not None:
                dst.copy_(torch.as_tensor(src, dtype=torch.float32).reshape(dst.shape))

    def launch(self):
        """Replay the graph on the current stream (no wait)."""
        self.graph.replay()

    def run(self, I=None, x=None, r=None, data=None):
        """(loss, gradient (N, P), Hessian (N, P, P) or None) as host tensors."""
        self.set_inputs(I, x, r, data)
        self.graph.replay()
        torch.cuda.current_stream(self.geom.device).synchronize()
        return float(self.loss_h), self.g_h, self.H_h


class FitLoop:
    """A whole damped-Newton fit as one CUDA graph (``gr_fit_loop_*``).

    ``capture_iteration()`` must issue one iteration on the current stream
    (projection + fit, derivatives, ``newton_solve_into``, trial projection,
    ``newton_accept_into``) with preallocated buffers only; it is captured
    into the body of a WHILE node.  After each iteration a device-side stop
    test reads ``hist``, ``hist_acc`` and ``counter`` (written by the accept
    kernel): it stops after ``max_iter`` iterations, after ``max_reject``
    rejected trials in a row, or when the last accepted iteration changed the
    loss by at most ``tol`` relative.  ``launch()`` runs the whole fit on
    ``stream`` with no host round trip.  ``close()`` waits for the device to
    idle (a property of destroying an executable graph): close finished loops
    when nothing runs.
    """

    def __init__(self, stream, capture_iteration, hist, hist_acc, counter, max_iter,
                 max_reject, tol, device, pass_loop=False):
        lib = _lib.load()
        self._lib = lib
        self.stream = stream
        self.handle = None
        self.guard = torch.zeros(1, dtype=torch.int32, device=device)
        self.stop_reason = torch.zeros(1, dtype=torch.int32, device=device)
        self._keep = (hist, hist_acc, counter)
        h = ctypes.c_void_p()
        sh = ctypes.c_void_p(stream.cuda_stream)
        import time
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            _lib.check(lib.gr_fit_loop_begin(sh, self.guard.data_ptr(), ctypes.byref(h)),
                       "gr_fit_loop_begin")
            self.handle = h
            t1 = time.perf_counter()
            try:
                if pass_loop:
                    capture_iteration(self)
                else:
                    capture_iteration()
            finally:
                t2 = time.perf_counter()
                rc = lib.gr_fit_loop_end(
                    h, sh, hist.data_ptr(), hist_acc.data_ptr(), counter.data_ptr(),
                    int(hist.numel()), int(max_iter), int(max_reject), float(tol),
                    int(max_iter) + int(max_reject) + 2, self.stop_reason.data_ptr())
        t3 = time.perf_counter()
        if rc == 0:
            rc = lib.gr_fit_loop_instantiate(h)
        # host seconds of each step of building the loop
        self.seconds = {"loop_begin": t1 - t0, "loop_iteration": t2 - t1,
                        "loop_end": t3 - t2, "loop_instantiate": time.perf_counter() - t3}
        if rc != 0:
            self.close()
            _lib.check(rc, "gr_fit_loop_end")

    @contextlib.contextmanager
    def unless_rejected(self):
        """During the capture (``pass_loop=True``): the work issued inside
        runs on an iteration only if the previous trial was accepted (or on
        the first iteration).  A rejected trial leaves the atoms and their
        fit fields unchanged, so derivatives issued here would reproduce
        the previous outputs bit for bit (``gr_fit_loop_gate_begin``)."""
        _hist, hist_acc, counter = self._keep
        sh = ctypes.c_void_p(self.stream.cuda_stream)
        _lib.check(self._lib.gr_fit_loop_gate_begin(self.handle, sh, hist_acc.data_ptr(),
                                                    counter.data_ptr(), int(hist_acc.numel())),
                   "gr_fit_loop_gate_begin")
        try:
            yield
        finally:
            _lib.check(self._lib.gr_fit_loop_gate_end(self.handle, sh), "gr_fit_loop_gate_end")

    def launch(self):
        _lib.check(self._lib.gr_fit_loop_launch(self.handle,
                                                ctypes.c_void_p(self.stream.cuda_stream)),
                   "gr_fit_loop_launch")

    def close(self):
        if self.handle is not None and self.handle.value:
            self._lib.gr_fit_loop_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchLoop:
    """Several small 2D L2 damped-Newton fits as one device loop
    (``gr_batch_*``): each kernel of an iteration is one launch over a table
    of the problems, and a problem leaves the loop when its own stop test
    (that of ``FitLoop``) says so.

    ``members``: objects with the device buffers of one fit each --
    ``cur``, ``trial`` (``DeviceAtoms``), ``geom``, ``data``, ``alpha_t``
    (the fit fields), ``loss_cur``, ``loss_trial``, ``theta``,
    ``theta_trial``, ``lam``, ``step``, ``f``, ``g``, ``H``, ``hist``,
    ``hist_acc``, ``counter`` and ``req`` (``max_iter``, ``tol``,
    ``lam_max``).  Raises ``EngineError`` when the members cannot share a
    batch (``gr_batch_workspace_bytes`` is 0).  ``launch()`` runs the
    prologue (fields and loss of every current atom set) and the loop on
    ``stream``."""

    def __init__(self, members, stream, setup_stream, device, max_reject, lam_min=1e-4):
        lib = _lib.load()
        self._lib = lib
        self.stream = stream
        self.handle = None
        self.batch = None
        n = len(members)
        arr = (_lib.GrBatchMember * n)()
        for a, m in zip(arr, members):
            a.cur = m.cur.struct
            a.trial = m.trial.struct
            a.geom = m.geom.struct
            a.data = m.data.data_ptr()
            a.fields = m.alpha_t.data_ptr()
            for name in ("loss_cur", "loss_trial", "theta", "theta_trial", "lam", "step", "f",
                         "g", "H", "hist", "counter"):
                setattr(a, name, getattr(m, name).data_ptr())
            a.hist_acc = m.hist_acc.data_ptr()
            a.hist_len = int(m.hist.numel())
            a.max_iter = int(m.req.max_iter)
            a.tol = float(m.req.tol)
            a.lam_min = float(lam_min)
            a.lam_max = float(m.req.lam_max)
        self._members = arr
        nb = int(lib.gr_batch_workspace_bytes(arr, n))
        if nb == 0:
            raise _lib.EngineError("these fits cannot share a batch")
        self.ws = torch.empty(nb, dtype=torch.uint8, device=device)
        h = ctypes.c_void_p()
        _lib.check(lib.gr_batch_create(arr, n, self.ws.data_ptr(), nb, int(max_reject),
                                       ctypes.c_void_p(setup_stream.cuda_stream),
                                       ctypes.byref(h)), "gr_batch_create")
        self.batch = h
        self.guard = torch.zeros(1, dtype=torch.int32, device=device)
        sh = ctypes.c_void_p(stream.cuda_stream)
        loop = ctypes.c_void_p()
        with torch.cuda.stream(stream):
            _lib.check(lib.gr_fit_loop_begin(sh, self.guard.data_ptr(), ctypes.byref(loop)),
                       "gr_fit_loop_begin")
            self.handle = loop
            rc = lib.gr_batch_iterate(self.batch, loop, sh)
            rc2 = lib.gr_fit_loop_end_open(loop, sh)
        if rc == 0:
            rc = rc2
        if rc == 0:
            rc = lib.gr_fit_loop_instantiate(loop)
        if rc != 0:
            self.close()
            _lib.check(rc, "gr_batch_iterate")

    def prologue(self):
        """Every member active; fit fields and loss of its current atoms."""
        sh = ctypes.c_void_p(self.stream.cuda_stream)
        _lib.check(self._lib.gr_batch_prologue(self.batch, sh), "gr_batch_prologue")

    def launch_loop(self):
        sh = ctypes.c_void_p(self.stream.cuda_stream)
        _lib.check(self._lib.gr_fit_loop_launch(self.handle, sh), "gr_fit_loop_launch")

    def launch(self):
        self.prologue()
        self.launch_loop()

    def close(self):
        if self.handle is not None and self.handle.value:
            self._lib.gr_fit_loop_destroy(self.handle)
        self.handle = None
        if self.batch is not None and self.batch.value:
            self._lib.gr_batch_destroy(self.batch)
        self.batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


REG_KINDS = {"null": 0, "joubert": 1, "mass": 2, "volume": 3, "radius": 4, "iso": 5}


def regulariser(kind, params, atoms, f=None, g=None, H=None, accumulate=False, order=2):
    """Per-atom regulariser value (N,), gradient (N, P) and Hessian (N, P, P)
    (order 2) in FP64 on the device (``gr_regulariser``); with
    ``accumulate=True`` the terms are added to the given f, g, H (e.g. the
    outputs of ``atom_derivs``).  ``kind`` is a name of ``REG_KINDS``."""
    import numpy as np
    dev = atoms.I.device
    n, P = atoms.n, atoms.n_params()
    f64 = dict(dtype=torch.float64, device=dev)
    if f is None:
        f = torch.zeros(n, **f64)
    if g is None:
        g = torch.zeros(n, P, **f64)
    if H is None and order > 1:
        H = torch.zeros(n, P, P, **f64)
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
    lib = _lib.load()
    st = lib.gr_regulariser(REG_KINDS[kind], p.ctypes.data if p.size else None, int(p.size),
                            ctypes.byref(atoms.struct), int(atoms.dim), _ptr(f), _ptr(g),
                            _ptr(H), 1 if accumulate else 0, _stream_handle(dev))
    _lib.check(st, "gr_regulariser")
    return f, g, H
