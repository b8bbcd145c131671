"""Autotuner for the derivative kernels' work split.

The derivative launch splits (atoms x angle chunks) into about
``GR_TUNE_DERIV_WARPS`` warps with at least ``GR_TUNE_DERIV_MIN_ANGLES`` angles
per lane group and ``GR_TUNE_DERIV_ATOMS_PER_WARP`` atoms per warp; the best split depends on the atom count, angle count,
support sizes and derivative order.  ``autotune_derivs`` times candidate
splits on the actual problem with CUDA events and keeps the fastest; results
are cached per shape class (detector dims, log2 atom count, log2 angle count,
order, pixel-integrated or not) and reapplied by ``apply_for``.
Results do not depend on the split beyond FP rounding of the chunk sums.
"""
import math

import torch

from . import _lib, engine

WARPS = (4096, 8192, 16384, 32768, 65536, 131072)
MIN_ANGLES = (1, 2, 4, 8)
ATOMS_PER_WARP = (1, 2, 4, 8)
_cache = {}


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
    """Time every candidate split on this problem; apply and return the best
    (target_warps, min_angles, atoms_per_warp, ms)."""
    key = shape_key(atoms, geom, order, psf)
    cands = candidates or [(w, m, g) for w in WARPS for m in MIN_ANGLES
                           for g in ATOMS_PER_WARP]
    saved = get_split()
    best = None
    for cand in cands:
        w, m = cand[0], cand[1]
        g = cand[2] if len(cand) > 2 else saved[2]
        set_split(w, m, g)
        engine.atom_derivs(atoms, geom, "field", field, beta_field, beta_const, order, psf=psf)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            engine.atom_derivs(atoms, geom, "field", field, beta_field, beta_const, order, psf=psf)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        if best is None or ms < best[3]:
            best = (w, m, g, ms)
    if best is None:
        set_split(*saved)
        return None
    _cache[key] = best[:3]
    set_split(*best[:3])
    return best


def apply_for(atoms, geom, order, psf=False):
    """Apply the cached split for this shape class, if any; returns it."""
    v = _cache.get(shape_key(atoms, geom, order, psf))
    if v is not None:
        set_split(*v)
    return v
