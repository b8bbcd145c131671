"""Seeded synthetic problems shared by the tests (reference geometry
conventions, GaussDictCode/atomFuncs.py:13-74)."""
import importlib

import numpy as np

from oracle import gauss_oracle as go

PKG = "2018_dictionary_tomography_gb300"


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def make_geometry(kind, A, D0, D1=None, det_box=1.5):
    """kind '2d', '2p5d' (single-axis tilt) or '3d' (two angle vectors)."""
    p0 = np.linspace(-det_box, det_box, D0)
    if kind == "2d":
        g = go.Geometry.from_angles([np.linspace(0, np.pi, A, endpoint=False)], p0)
    elif kind == "2p5d":
        p1 = np.linspace(-det_box, det_box, D1 or D0)
        g = go.Geometry.from_angles([np.linspace(-np.pi / 3, np.pi / 3, A)], p0, p1)
    elif kind == "3d":
        a0 = int(np.ceil(np.sqrt(A)))
        a1 = max(1, A // a0)
        p1 = np.linspace(-det_box, det_box, D1 or D0)
        g = go.Geometry.from_angles([np.linspace(0.1, np.pi, a0, endpoint=False),
                                     np.linspace(-1.0, 1.2, a1)], p0, p1)
    else:
        raise ValueError(kind)
    # the engine consumes float32 geometry: give the oracle the same values
    return g.cast(np.float32).cast(np.float64)


def make_atoms(dim, N, seed, iso=False, rdiag=(3.0, 6.0), roff=1.0, box=0.5,
               Irange=(0.5, 1.5)):
    rng = np.random.default_rng(seed)
    I = rng.uniform(*Irange, N)
    x = rng.uniform(-box, box, (N, dim))
    if iso:
        r = rng.uniform(*rdiag, (N, 1))
    else:
        pr = 3 if dim == 2 else 6
        r = np.concatenate([rng.uniform(*rdiag, (N, dim)),
                            rng.normal(0, roff, (N, pr - dim))], axis=1)
    return f32(I), f32(x), f32(r)


def engine_geometry(g):
    geometry = importlib.import_module(PKG + ".geometry")
    if g.gm == 2:
        return geometry.DeviceGeometry(g.T, (g.w0,), [g.p0])
    if g.gm == 25:
        return geometry.DeviceGeometry(g.T, (g.w0,), [g.p0, g.p1])
    return geometry.DeviceGeometry(g.T, (g.w0, g.w1), [g.p0, g.p1])


def engine_atoms(I, x, r):
    engine = importlib.import_module(PKG + ".engine")
    return engine.DeviceAtoms(I, x, r)


def relerr(a, ref):
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.max(np.abs(ref))
    if scale == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - ref)) / scale)


def entry_relerr(a, ref):
    """Max error per parameter entry (or entry pair), scaled by that entry's
    largest magnitude over all atoms; entries whose reference is zero for
    every atom are scaled by the overall maximum."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    tot = np.max(np.abs(ref))
    scale = np.max(np.abs(ref), axis=0)
    scale = np.where(scale > 1e-9 * tot, scale, tot)
    return float(np.max(np.abs(a - ref) / scale))


def atom_normwise_relerr(a, ref):
    """Max over atoms of max|a_j - ref_j| / max|ref_j| (each atom's matrix
    scaled by its own largest entry)."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    n = ref.shape[0]
    d = np.abs(a - ref).reshape(n, -1).max(axis=1)
    sc = np.abs(ref).reshape(n, -1).max(axis=1)
    sc = np.where(sc > 0, sc, 1.0)
    return float(np.max(d / sc))
