"""Python front of the Gaussian-atom Radon oracle.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the product path never
does.  It wraps the C restatement in ``oracle_impl.h`` (FP64 oracle and FP32
twin) and adds:

* geometry restated from the reference (``theta_to_vec`` / ``perp``,
  GaussDictCode/atomFuncs.py:13-74);
* the isotropic rule: an isotropic atom ``r = s`` is the anisotropic atom
  ``r = (s, s, 0)`` (2D) or ``(s, s, s, 0, 0, 0)`` (3D), and its derivatives are
  the exact chain rule of that map (sum of the diagonal-r rows/columns).  This
  is the corrected form of the reference's collapse
  (GaussDictCode/bin/NewtonBases2D.py:319-324, :435-440), which indexes out of
  range in 2D and omits the 2*H[3,4] cross term;
* the all-atoms data-fit derivatives used by the Newton/GD loops: for atom j
  the reference calls ``L2derivs_RadProj(atom_j, Rad, data + R_j - R_total)``
  (NewtonGaussian.py:59-60), which this module evaluates for every atom.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = ctypes.CDLL(path)
        for sfx in ("_f64", "_f32"):
            getattr(_lib, "or_radproj" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_radproj_boxed" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_atom_derivs_boxed" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_atom_derivs" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_point_derivs" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_volproj" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_count_support" + sfx).restype = ctypes.c_longlong
            getattr(_lib, "or_psf_radproj" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_psf_atom_derivs" + sfx).restype = ctypes.c_int
            getattr(_lib, "or_psf_volproj" + sfx).restype = ctypes.c_int
    return _lib


def _nthreads(n):
    return int(n) if n else (os.cpu_count() or 1)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


# --------------------------------------------------------------------------
# geometry (restated from GaussDictCode/atomFuncs.py:13-74)
# --------------------------------------------------------------------------
def theta_to_vec(theta):
    """Ray directions T for one (2D) or two (3D) angle vectors."""
    theta = [np.asarray(t, dtype=np.float64) for t in theta]
    if len(theta) == 1:
        t = theta[0]
        return np.stack([-np.sin(t), np.cos(t)], axis=-1)
    t0, t1 = np.meshgrid(theta[0], theta[1], indexing="ij")
    return np.stack([-np.sin(t0) * np.cos(t1), np.cos(t0) * np.cos(t1),
                     np.sin(t1)], axis=-1)


def perp(theta):
    """Detector axes perpendicular to theta_to_vec(theta)."""
    theta = [np.asarray(t, dtype=np.float64) for t in theta]
    if len(theta) == 1:
        t = theta[0]
        return (np.stack([np.cos(t), np.sin(t)], axis=-1),)
    t0, t1 = np.meshgrid(theta[0], theta[1], indexing="ij")
    o0 = np.stack([np.cos(t0), np.sin(t0), np.zeros_like(t0)], axis=-1)
    o1 = np.stack([np.sin(t0) * np.sin(t1), -np.cos(t0) * np.sin(t1),
                   np.cos(t1)], axis=-1)
    return o0, o1


class Geometry:
    """Flat geometry arrays in the reference's layout.

    gm = 2 (2D), 3 (3D, two detector axes w0/w1) or 25 (2.5D single-axis
    tilt: T and w0 have two components and the second detector axis is the
    atom coordinate 2).
    """

    def __init__(self, gm, T, w0, p0, w1=None, p1=None):
        self.gm = int(gm)
        self.T = np.ascontiguousarray(T, dtype=np.float64)
        self.w0 = np.ascontiguousarray(w0, dtype=np.float64)
        self.w1 = None if w1 is None else np.ascontiguousarray(w1, dtype=np.float64)
        self.p0 = np.ascontiguousarray(p0, dtype=np.float64).reshape(-1)
        self.p1 = None if p1 is None else np.ascontiguousarray(p1, dtype=np.float64).reshape(-1)
        self.A = self.T.shape[0]
        self.dim = 2 if self.gm == 2 else 3
        self.shape = (self.A, self.p0.size) if self.gm == 2 else (self.A, self.p0.size, self.p1.size)

    @staticmethod
    def from_angles(angles, det0, det1=None):
        """angles: list of one (2D / 2.5D) or two (3D) angle vectors."""
        T = theta_to_vec(angles).reshape(-1, len(angles) + 1)
        w = [o.reshape(-1, len(angles) + 1) for o in perp(angles)]
        if len(angles) == 1 and det1 is None:
            return Geometry(2, T, w[0], det0)
        if len(angles) == 1:
            return Geometry(25, T, w[0], det0, None, det1)
        return Geometry(3, T, w[0], det0, w[1], det1)

    def cast(self, dtype):
        g = Geometry.__new__(Geometry)
        g.__dict__.update(self.__dict__)
        for k in ("T", "w0", "w1", "p0", "p1"):
            v = getattr(self, k)
            setattr(g, k, None if v is None else np.ascontiguousarray(v, dtype=dtype))
        return g


def _dims(dim):
    pr = 3 if dim == 2 else 6
    return pr, 1 + dim + pr


def to_aniso(r, dim):
    r = np.asarray(r, dtype=np.float64)
    r = r.reshape(r.shape[0], -1)
    pr, _ = _dims(dim)
    if r.shape[1] == pr:
        return r.copy()
    out = np.zeros((r.shape[0], pr))
    out[:, :dim] = r[:, :1]
    return out


def collapse_iso(df, ddf, dim):
    """Exact chain rule for r_aniso = (s,..,s,0,..): J sums the diagonal-r
    entries.  df: (..., P_aniso), ddf: (..., P_aniso, P_aniso)."""
    _, P = _dims(dim)
    J = np.zeros((P, 2 + dim))
    for i in range(1 + dim):
        J[i, i] = 1
    J[1 + dim:1 + 2 * dim, 1 + dim] = 1
    dfi = df @ J
    ddfi = None if ddf is None else np.einsum("...ij,ia,jb->...ab", ddf, J, J)
    return dfi, ddfi


# --------------------------------------------------------------------------
# wrappers
# --------------------------------------------------------------------------
def radproj(I, x, r, geom, dtype=np.float64, nthreads=None):
    """Dense forward projection (every atom at every cell)."""
    dim = geom.dim
    g = geom.cast(dtype)
    I = np.ascontiguousarray(I, dtype=dtype).reshape(-1)
    x = np.ascontiguousarray(x, dtype=dtype).reshape(-1, dim)
    r = np.ascontiguousarray(to_aniso(r, dim), dtype=dtype)
    out = np.zeros(geom.shape, dtype=dtype)
    fn = lib().or_radproj_f64 if dtype == np.float64 else lib().or_radproj_f32
    D1 = 1 if dim == 2 else g.p1.size
    rc = fn(g.gm, I.size, _p(I), _p(x), _p(r), g.A, _p(g.T), _p(g.w0), _p(g.w1),
            g.p0.size, _p(g.p0), D1, _p(g.p1), _p(out), _nthreads(nthreads))
    assert rc == 0
    return out


def radproj_boxed(I, x, r, geom, dtype=np.float64, nthreads=None):
    """radproj visiting only each atom's shadow box per angle (same result:
    every cell outside the boxes is exactly zero in the dense sum)."""
    dim = geom.dim
    g = geom.cast(dtype)
    I = np.ascontiguousarray(I, dtype=dtype).reshape(-1)
    x = np.ascontiguousarray(x, dtype=dtype).reshape(-1, dim)
    r = np.ascontiguousarray(to_aniso(r, dim), dtype=dtype)
    out = np.empty(geom.shape, dtype=dtype)
    fn = lib().or_radproj_boxed_f64 if dtype == np.float64 else lib().or_radproj_boxed_f32
    D1 = 1 if dim == 2 else g.p1.size
    rc = fn(g.gm, I.size, _p(I), _p(x), _p(r), g.A, _p(g.T), _p(g.w0), _p(g.w1),
            g.p0.size, _p(g.p0), D1, _p(g.p1), _p(out), _nthreads(nthreads))
    assert rc == 0
    return out


def atom_derivs(kind, I, x, r, geom, C, order=2, dtype=np.float64, nthreads=None,
                beta=None, boxed=False):
    """Single-atom derivatives summed over all cells.

    kind "l2": of 1/2|R(atom) - C|^2;  kind "ip": of <R(atom), C>;
    kind "field": g = sum C dR, H = sum beta dR dR^T + C ddR (C = alpha).
    r may be isotropic (one entry); results then use the exact chain rule.
    Returns (f, Df (P,), DDf (P,P)) in float64.
    """
    dim = geom.dim
    g = geom.cast(dtype)
    r_in = np.asarray(r, dtype=np.float64).reshape(-1)
    iso = r_in.size == 1
    ra = np.ascontiguousarray(to_aniso(r_in.reshape(1, -1), dim).reshape(-1), dtype=dtype)
    I = np.ascontiguousarray(np.reshape(I, -1)[:1], dtype=dtype)
    x = np.ascontiguousarray(np.reshape(x, -1)[:dim], dtype=dtype)
    C = np.ascontiguousarray(C, dtype=dtype).reshape(geom.shape)
    B = None
    if kind == "field":
        B = np.ascontiguousarray(beta, dtype=dtype).reshape(geom.shape)
    _, P = _dims(dim)
    f = np.zeros(1)
    Df = np.zeros(P)
    DDf = np.zeros(P * P)
    code = {"l2": 0, "ip": 1, "field": 2}[kind]
    if boxed and code == 0:
        raise ValueError("boxed evaluation covers the 'ip' and 'field' kinds")
    name = "or_atom_derivs_boxed" if boxed else "or_atom_derivs"
    fn = getattr(lib(), name + ("_f64" if dtype == np.float64 else "_f32"))
    D1 = 1 if dim == 2 else g.p1.size
    rc = fn(code, g.gm, _p(I), _p(x), _p(ra), g.A, _p(g.T),
            _p(g.w0), _p(g.w1), g.p0.size, _p(g.p0), D1, _p(g.p1), _p(C), _p(B),
            int(order), _p(f), _p(Df), _p(DDf), _nthreads(nthreads))
    assert rc == 0
    DDf = DDf.reshape(P, P)
    if iso:
        Df, DDf = collapse_iso(Df, DDf, dim)
    return f[0], Df, DDf


def all_atom_derivs(kind, I, x, r, geom, C, order=2, dtype=np.float64, nthreads=None,
                    beta=None):
    """atom_derivs for every atom (kind "ip": <R(atom_j), C>; kind "l2fit":
    the Newton-loop call L2derivs(atom_j, data + R_j - R_total) with
    C = data; kind "l2": each atom alone fitted to C; kind "field": weight
    fields C = alpha and beta)."""
    I = np.asarray(I, dtype=np.float64).reshape(-1)
    x = np.asarray(x, dtype=np.float64).reshape(I.size, -1)
    r = np.asarray(r, dtype=np.float64).reshape(I.size, -1)
    if kind == "l2fit":
        Rtot = radproj(I, x, r, geom, dtype=np.float64, nthreads=nthreads)
    fs, dfs, ddfs = [], [], []
    for j in range(I.size):
        if kind == "l2fit":
            Rj = radproj(I[j:j + 1], x[j:j + 1], r[j:j + 1], geom, nthreads=nthreads)
            Cj = np.asarray(C, dtype=np.float64) + Rj - Rtot
            out = atom_derivs("l2", I[j], x[j], r[j], geom, Cj, order, dtype, nthreads)
        else:
            out = atom_derivs(kind, I[j], x[j], r[j], geom, C, order, dtype, nthreads,
                              beta=beta)
        fs.append(out[0])
        dfs.append(out[1])
        ddfs.append(out[2])
    return np.array(fs), np.array(dfs), np.array(ddfs)


def count_support(x, r, geom, nthreads=None):
    """Dense count of (atom, angle, cell) triples with m <= 1."""
    dim = geom.dim
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, dim)
    r = np.ascontiguousarray(to_aniso(r, dim), dtype=np.float64)
    I = np.ones(x.shape[0])
    D1 = 1 if dim == 2 else geom.p1.size
    return int(lib().or_count_support_f64(
        geom.gm, x.shape[0], _p(I), _p(x), _p(r), geom.A, _p(geom.T), _p(geom.w0),
        _p(geom.w1), geom.p0.size, _p(geom.p0), D1, _p(geom.p1), _nthreads(nthreads)))


def point_derivs(dim, lenT, I, x, r, y, T, order=2):
    """Per-point value, gradient (P) and Hessian (P,P) in FP64."""
    _, P = _dims(dim)
    ra = np.ascontiguousarray(np.asarray(r, dtype=np.float64).reshape(-1))
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.pad(np.asarray(y, dtype=np.float64), (0, 3 - len(y))))
    T = np.ascontiguousarray(np.pad(np.asarray(T, dtype=np.float64), (0, 3 - len(T))))
    R = np.zeros(1)
    dR = np.zeros(P)
    ddR = np.zeros(P * P)
    lib().or_point_derivs_f64(dim, lenT, ctypes.c_double(float(I)), _p(x), _p(ra),
                              _p(y), _p(T), _p(R), _p(dR), _p(ddR), int(order))
    return R[0], dR, ddR.reshape(P, P)


def volproj(I, x, r, coords, dtype=np.float64, nthreads=None):
    """Render atoms on the voxel grid given by coordinate vectors."""
    dim = len(coords)
    I = np.ascontiguousarray(I, dtype=dtype).reshape(-1)
    x = np.ascontiguousarray(x, dtype=dtype).reshape(-1, dim)
    r = np.ascontiguousarray(to_aniso(r, dim), dtype=dtype)
    ys = [np.ascontiguousarray(c, dtype=dtype).reshape(-1) for c in coords]
    if dim == 2:
        ys.append(np.zeros(1, dtype=dtype))
    out = np.zeros([y.size for y in ys[:dim]], dtype=dtype)
    fn = lib().or_volproj_f64 if dtype == np.float64 else lib().or_volproj_f32
    rc = fn(dim, I.size, _p(I), _p(x), _p(r), ys[0].size, _p(ys[0]), ys[1].size,
            _p(ys[1]), ys[2].size, _p(ys[2]), _p(out), _nthreads(nthreads))
    assert rc == 0
    return out


def l2_value(R, data):
    """1/2 sum (R - data)^2 (GaussDictCode/transport_loss.py:569-585)."""
    d = np.asarray(R, dtype=np.float64) - np.asarray(data, dtype=np.float64)
    return 0.5 * float(np.sum(d * d))


def kl_value(f, R, b):
    """KL(f || R + b) = sum f log(f/(R+b)) - f + (R+b), with 0 log 0 = 0.

    The reference's KL_2D (KL_GaussRadon.py:52-54) is nansum(f (log(f/g) - 1)
    + g); the background b > 0 keeps g positive where atoms have no support.
    """
    f = np.asarray(f, dtype=np.float64)
    g = np.asarray(R, dtype=np.float64) + b
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(f > 0, f * np.log(f / g), 0.0)
    return float(np.sum(t - f + g))


def kl_fields(f, R, b):
    """Per-pixel weights of the KL derivatives: alpha = 1 - f/g (first order),
    beta = f/g^2 (Gauss-Newton)."""
    f = np.asarray(f, dtype=np.float64)
    g = np.asarray(R, dtype=np.float64) + b
    return 1.0 - f / g, f / (g * g)


# --------------------------------------------------------------------------
# single-particle (pixel-integrated) operator
# --------------------------------------------------------------------------
def psf_radproj(I, x, r, geom, dtype=np.float64, nthreads=None):
    """Pixel-integrated projection (point_spread_functions.RadProj)."""
    dim = geom.dim
    g = geom.cast(dtype)
    I = np.ascontiguousarray(I, dtype=dtype).reshape(-1)
    x = np.ascontiguousarray(x, dtype=dtype).reshape(-1, dim)
    r = np.ascontiguousarray(to_aniso(r, dim), dtype=dtype)
    out = np.zeros(geom.shape, dtype=dtype)
    fn = lib().or_psf_radproj_f64 if dtype == np.float64 else lib().or_psf_radproj_f32
    D1 = 1 if dim == 2 else g.p1.size
    rc = fn(g.gm, I.size, _p(I), _p(x), _p(r), g.A, _p(g.T), _p(g.w0), _p(g.w1),
            g.p0.size, _p(g.p0), D1, _p(g.p1), _p(out), _nthreads(nthreads))
    assert rc == 0
    return out


def psf_atom_derivs(kind, I, x, r, geom, C, order=2, nthreads=None):
    """Single-atom derivatives of the pixel-integrated projection:
    kind "l2" (L2derivs_RadProj) or "ip" (derivs_RadProj); isotropic r uses
    the exact chain rule."""
    dim = geom.dim
    r_in = np.asarray(r, dtype=np.float64).reshape(-1)
    iso = r_in.size == 1
    ra = np.ascontiguousarray(to_aniso(r_in.reshape(1, -1), dim).reshape(-1))
    I = np.ascontiguousarray(np.reshape(I, -1)[:1], dtype=np.float64)
    x = np.ascontiguousarray(np.reshape(x, -1)[:dim], dtype=np.float64)
    C = np.ascontiguousarray(C, dtype=np.float64).reshape(geom.shape)
    _, P = _dims(dim)
    f = np.zeros(1)
    Df = np.zeros(P)
    DDf = np.zeros(P * P)
    D1 = 1 if dim == 2 else geom.p1.size
    rc = lib().or_psf_atom_derivs_f64(0 if kind == "l2" else 1, geom.gm, _p(I), _p(x), _p(ra),
                                      geom.A, _p(geom.T), _p(geom.w0), _p(geom.w1),
                                      geom.p0.size, _p(geom.p0), D1, _p(geom.p1), _p(C),
                                      int(order), _p(f), _p(Df), _p(DDf), _nthreads(nthreads))
    assert rc == 0
    DDf = DDf.reshape(P, P)
    if iso:
        Df, DDf = collapse_iso(Df, DDf, dim)
    return f[0], Df, DDf


def psf_volproj(I, x, r, coords, nthreads=None):
    """Voxel-integrated rendering (point_spread_functions.VolProj)."""
    dim = len(coords)
    I = np.ascontiguousarray(I, dtype=np.float64).reshape(-1)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, dim)
    r = np.ascontiguousarray(to_aniso(r, dim), dtype=np.float64)
    ys = [np.ascontiguousarray(c, dtype=np.float64).reshape(-1) for c in coords]
    if dim == 2:
        ys.append(np.zeros(1))
    out = np.zeros([y.size for y in ys[:dim]])
    rc = lib().or_psf_volproj_f64(dim, I.size, _p(I), _p(x), _p(r), ys[0].size, _p(ys[0]),
                                  ys[1].size, _p(ys[1]), ys[2].size, _p(ys[2]), _p(out),
                                  _nthreads(nthreads))
    assert rc == 0
    return out
