"""Autotuner for the derivative kernels' work split.

The derivative launch splits (atoms x angle chunks) into about
``GR_TUNE_DERIV_WARPS`` warps with at least ``GR_TUNE_DERIV_MIN_ANGLES`` angles
per lane group and ``GR_TUNE_DERIV_ATOMS_PER_WARP`` atoms per warp; the best split depends on the atom count, angle count,
support sizes and derivative order.  ``autotune_derivs`` times candidate
splits on the actual problem with CUDA events and keeps the fastest as an
``engine.Plan`` (the C ABI's gr_plan) cached per shape class (detector dims,
log2 atom count, log2 angle count, order, pixel-integrated or not):
``plan_for`` returns it, and launches given that plan run the tuned split
while other streams keep theirs; the process-wide values are not touched.
Results do not depend on the split beyond FP rounding of the chunk sums.
"""
import math

import torch

from . import _lib, engine

WARPS = (4096, 8192, 16384, 32768, 65536, 131072)
MIN_ANGLES = (1, 2, 4, 8)
ATOMS_PER_WARP = (1, 2, 4, 8)
_cache = {}
MARGIN = 0.03   # relative time a candidate must save to replace an earlier one


def set_split(target_warps, min_angles, atoms_per_warp=None):
    lib = _lib.load()
    _lib.check(lib.gr_set_tuning(0, int(target_warps)), "gr_set_tuning")
    _lib.check(lib.gr_set_tuning(1, int(min_angles)), "gr_set_tuning")
    if atoms_per_warp is not None:
        _lib.check(lib.gr_set_tuning(2, int(atoms_per_warp)), "gr_set_tuning")


def set_projection_tiling(form):
    """1: 16 x 32-cell tiles (default), 2: 32 x 32 (3D point-sampled
    projection)."""
    _lib.check(_lib.load().gr_set_tuning(3, int(form)), "gr_set_tuning")


def set_projection_split(cells):
    """3D problems with fewer detector cells (all angles) than ``cells``
    split each tile's atoms over a block's warps (0: never)."""
    _lib.check(_lib.load().gr_set_tuning(4, int(cells)), "gr_set_tuning")


def set_derivative_split(lanes):
    """Problems with fewer (atom, angle) pairs than ``lanes`` split each
    pair's cells over 2, 4 or 8 lanes of the derivative kernel (0: never)."""
    _lib.check(_lib.load().gr_set_tuning(6, int(lanes)), "gr_set_tuning")


def set_one_angle_budget(mb):
    """Give every derivative lane at most one angle whenever the chunk
    partials then fit in ``mb`` MB (0: keep the target-warps split)."""
    _lib.check(_lib.load().gr_set_tuning(7, int(mb)), "gr_set_tuning")


def get_one_angle_budget():
    return int(_lib.load().gr_get_tuning(7))


def get_derivative_split():
    return int(_lib.load().gr_get_tuning(6))


def get_projection_split():
    return int(_lib.load().gr_get_tuning(4))


def get_split():
    lib = _lib.load()
    return int(lib.gr_get_tuning(0)), int(lib.gr_get_tuning(1)), int(lib.gr_get_tuning(2))


def shape_key(atoms, geom, order, psf=False):
    return (geom.kdet, int(math.log2(max(1, atoms.n))), int(math.log2(max(1, geom.n_angles))),
            int(order), bool(psf))


def autotune_derivs(atoms, geom, field, beta_field=None, beta_const=1.0, order=1,
                    psf=False, reps=5, candidates=None):
    """Time every candidate split on this problem under a plan of its own;
    cache the best plan for the problem's shape class and return
    (target_warps, min_angles, atoms_per_warp, ms).  The process-wide
    schedule is left as it was."""
    key = shape_key(atoms, geom, order, psf)
    cands = candidates or [(w, m, g) for w in WARPS for m in MIN_ANGLES
                           for g in ATOMS_PER_WARP]
    op = _lib.GR_OP_DERIVS_1 if order == 1 else _lib.GR_OP_DERIVS_2
    plan = engine.Plan(op, atoms, geom)
    best = None
    for cand in cands:
        w, m = cand[0], cand[1]
        g = cand[2] if len(cand) > 2 else plan.get(2)
        wide = cand[3] if len(cand) > 3 else 0
        plan.set(0, w).set(1, m).set(2, g).set(8, wide)
        run = lambda: engine.atom_derivs(atoms, geom, "field", field, beta_field, beta_const,
                                         order, psf=psf, plan=None if psf else plan)
        if psf:
            # the pixel-integrated kernels run under the process-wide values
            saved = get_split()
            set_split(w, m, g)
        run()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            run()
        b.record()
        torch.cuda.synchronize()
        if psf:
            set_split(*saved)
        ms = a.elapsed_time(b) / reps
        # the first candidate is kept unless another is clearly faster: a
        # split timed alone on an idle GPU that wins by a hair need not win
        # among concurrent fits
        if best is None or ms < best[3] * (1.0 - MARGIN):
            best = (w, m, g, ms, wide)
    if best is None:
        return None
    plan.set(0, best[0]).set(1, best[1]).set(2, best[2]).set(8, best[4])
    _cache[key] = plan
    return best[:4]


def plan_for(atoms, geom, order, psf=False):
    """The tuned plan of this shape class, or None (then the process-wide
    schedule applies)."""
    return _cache.get(shape_key(atoms, geom, order, psf))


def apply_for(atoms, geom, order, psf=False):
    """The cached split (target_warps, min_angles, atoms_per_warp) of this
    shape class, or None; use ``plan_for`` to run under it."""
    p = plan_for(atoms, geom, order, psf)
    return None if p is None else (p.get(0), p.get(1), p.get(2))


# ---------------------------------------------------------------------------
# serving: plans per shape class of fitting requests
# ---------------------------------------------------------------------------
_req_plans = {}
# small candidate sets: a server tunes each new class once, on its first
# request, and the fits of the class then run under the winners
# (only the row-walk switch for the derivatives: splits into fewer warps won
# alone on an idle GPU but lost among concurrent fits, 1.655 s against 1.624 s
# untuned on the 512-request stream)
DERIV_CANDIDATES = ((131072, 1, 1, 0), (131072, 1, 1, 1))
PROJ_CANDIDATES = ((1, 4 << 20), (1, 0), (2, 4 << 20), (2, 0))
# 2D: the block split does not apply; tiles of 32, 64 or 128 cells
PROJ_CANDIDATES_2D = ((1, 0), (2, 0), (3, 0))


def request_key(req, order=2):
    """Shape class of a fitting request (as shape_key)."""
    n = len(req.init[0])
    return (len(req.detector), int(math.log2(max(1, n))),
            int(math.log2(max(1, len(req.orientations)))), int(order), False)


def plans_for_request(req, order=2):
    """(projection plan, derivative plan) of the request's class, or
    (None, None) when the class has not been tuned."""
    return _req_plans.get(request_key(req, order), (None, None))


def tune_request_classes(requests, device, reps=3, order=2):
    """Tune each shape class among ``requests`` once, on its first request:
    the projection's tiling and block split and the derivative split, each
    timed under a plan of its own.  Returns the number of classes tuned."""
    from .geometry import DeviceGeometry
    done = 0
    for req in requests:
        key = request_key(req, order)
        if key in _req_plans:
            continue
        geom = DeviceGeometry(req.orientations, req.ortho, req.detector, device)
        atoms = engine.DeviceAtoms(*req.init, device)
        stream = torch.cuda.current_stream(device)
        data = req.device_data(geom, device, stream)
        pp = engine.Plan(_lib.GR_OP_PROJECT, atoms, geom)
        best_p = None
        for form, split in (PROJ_CANDIDATES_2D if len(req.detector) == 1 else PROJ_CANDIDATES):
            pp.set(3, form).set(4, split)
            ms = _time(lambda: engine.fit_forward(atoms, geom, data, req.fit, req.background,
                                                  plan=pp), reps)
            if best_p is None or ms < best_p[2] * (1.0 - MARGIN):
                best_p = (form, split, ms)
        pp.set(3, best_p[0]).set(4, best_p[1])
        fw = engine.fit_forward(atoms, geom, data, req.fit, req.background, plan=pp)
        autotune_derivs(atoms, geom, fw["alpha"], fw["beta"],
                        1.0 if req.fit == "l2" else 0.0, order=order, reps=reps,
                        candidates=DERIV_CANDIDATES)
        _req_plans[key] = (pp, plan_for(atoms, geom, order))
        done += 1
    torch.cuda.synchronize(device)
    return done


def _time(fn, reps):
    fn()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps
