"""Golden vectors computed by the reference's own kernel and fitting code.

Loads, by path and under the CPU stand-in for numba in ``ref_numba_stub.py``:

* GaussDictCode/bin/{numba_cuda_aux,NewtonBases,NewtonBases2D,
  point_spread_functions,manager}.py and GaussDictCode/{transport_loss,
  regularisation}.py (the kernel modules, the array context, the L2 loss);
* NewtonGaussian.py and GD_lib.py (the fitting loops; matplotlib and skimage,
  used there for plotting only, are replaced by no-op modules).

The package ``__init__`` files are bypassed (they import odl and spyder).  The
kernels run through the stub's SIMT emulation in FP64 (the reference's ``f4``
local/shared arrays and its host ``empty(..., dtype='f4')`` output buffers are
made float64), so the outputs are the reference's arithmetic in double
precision.  The host wrappers are called exactly as the reference's
``GaussTomo`` calls them (GaussDictCode/atomFuncs.py:115-158), with duck-typed
atom and space objects carrying the attributes the wrappers read.

What is recorded (``tests/golden/reference_kernels.npz``):

* per-cell ``__Rf``/``__dRf`` (NewtonBases2D.py:39-243) and
  ``__Rf``/``__dRf_aniso`` (NewtonBases.py:262-528) with the 3D and 2.5D cell
  maps ``__tovec3D``/``__tovec2p5D`` (NewtonBases.py:677-688);
* ``RadProj``, ``L2derivs_RadProj`` and ``derivs_RadProj`` (order 2) of the 2D,
  2.5D and 3D modules on small seeded problems, and ``VolProj``;
* the pixel-integrated module's ``RadProj``, ``L2derivs_RadProj``,
  ``derivs_RadProj`` and ``VolProj`` (point_spread_functions.py:143-1523) in 2D
  and 3D;
* ``NewtonGaussian.linesearch`` and ``GD_lib.linesearch_block`` runs on a small
  2D anisotropic L2 problem: final atoms and the energy history;
* ``KL_GaussRadon.doKL_ProjGDStep_iso`` (the moment-matching atom guess) on a
  seeded 2D residual with t = 1 and t = 0.5.

Needs the reference checkout (run from the repository root):

    python tests/golden/make_ref_golden.py /root/reference
"""
import importlib
import importlib.util
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_numba_stub  # noqa: E402

F64 = np.float64


# ---------------------------------------------------------------------------
# loading
# ---------------------------------------------------------------------------
def _f4_to_f64(fn):
    def wrapped(*a, **kw):
        dt = kw.get("dtype")
        if len(a) > 1 and not isinstance(a[1], (list, tuple)) and a[1] in ("f4", "float32"):
            a = (a[0], F64) + a[2:]
        if dt in ("f4", "float32"):
            kw["dtype"] = F64
        return fn(*a, **kw)
    return wrapped


class _Anything:
    """No-op object for the plotting calls of GD_lib._startup."""

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()

    def __getitem__(self, k):
        return _Anything()

    def __iter__(self):
        return iter((_Anything(), _Anything()))


def load_reference(root):
    ref_numba_stub.install()
    # plotting-only imports of GD_lib / NewtonGaussian
    skimage = types.ModuleType("skimage")
    skimage.measure = _Anything()
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.subplots = lambda *a, **k: (_Anything(), _Anything())
    for name in ("draw", "pause", "show"):
        setattr(plt, name, lambda *a, **k: None)
    mpl.pyplot = plt
    sys.modules.update({"skimage": skimage, "matplotlib": mpl, "matplotlib.pyplot": plt})
    # names numpy 2 removed and the reference still imports
    if not hasattr(np, "infty"):
        np.infty = np.inf
    import warnings
    np.warnings = warnings
    sys.modules.setdefault("numpy.linalg.linalg", np.linalg)

    pkg = types.ModuleType("GaussDictCode")
    pkg.__path__ = [os.path.join(root, "GaussDictCode")]
    binpkg = types.ModuleType("GaussDictCode.bin")
    binpkg.__path__ = [os.path.join(root, "GaussDictCode", "bin")]
    pkg.bin = binpkg
    sys.modules.update({"GaussDictCode": pkg, "GaussDictCode.bin": binpkg})
    mods = {}
    for name in ("numba_cuda_aux", "NewtonBases", "NewtonBases2D", "point_spread_functions",
                 "manager"):
        mods[name] = importlib.import_module("GaussDictCode.bin." + name)
    for name in ("transport_loss", "regularisation"):
        mods[name] = importlib.import_module("GaussDictCode." + name)
    for name in ("NewtonBases", "NewtonBases2D", "point_spread_functions"):
        m = mods[name]
        for fn in ("empty", "zeros", "array"):
            if hasattr(m, fn):
                setattr(m, fn, _f4_to_f64(getattr(m, fn)))
    sys.path.insert(0, root)
    for name in ("GD_lib", "NewtonGaussian"):
        spec = importlib.util.spec_from_file_location("ref_" + name,
                                                      os.path.join(root, name + ".py"))
        m = importlib.util.module_from_spec(spec)
        sys.modules["ref_" + name] = m
        if name == "NewtonGaussian":
            sys.modules["GD_lib"] = mods["GD_lib"]
        spec.loader.exec_module(m)
        mods[name] = m
    # the plotter of GD_lib._startup draws views of the atoms: nothing to draw here
    for fn in ("_plot2D", "_plot2DwithGT", "_plot3D", "_plot3DwithGT"):
        setattr(mods["GD_lib"], fn, lambda *a, **k: None)
    return mods


def dev(mod, name):
    """A module-level device function whose name starts with two underscores."""
    return mod.__dict__[name]


# ---------------------------------------------------------------------------
# duck types with the attributes the reference's wrappers and loops read
# ---------------------------------------------------------------------------
class NS:
    def __init__(self, **kw):
        self.__dict__.update(kw)


class Atoms:
    """Like dictionary_def.AtomElement: arrays I (N,), x (N,d), r (N,k) in the
    context's float type; indexing returns a copy (AtomElement.__getitem__
    builds a new element through context().cast)."""

    def __init__(self, dim, iso, I, x, r):
        self.space = NS(dim=dim, isotropic=iso)
        self.I = np.array(I, dtype=F64).reshape(-1)
        self.x = np.array(x, dtype=F64).reshape(self.I.size, dim)
        self.r = np.array(r, dtype=F64).reshape(self.I.size, -1)
        self.size = self.I.size

    def __len__(self):
        return self.size

    def __getitem__(self, i):
        return Atoms(self.space.dim, self.space.isotropic, np.atleast_1d(self.I[i]),
                     self.x[i], self.r[i])


class Sino(np.ndarray):
    """Stands in for a ProjElement: ``.data``/``.asarray()`` give the array."""

    @property
    def data(self):
        return self.view(np.ndarray)

    def asarray(self):
        return self.view(np.ndarray)


class Tomo:
    """The reference's GaussTomo call protocol (atomFuncs.py:115-158) around a
    kernel module's four callables."""

    def __init__(self, mod, T, w, p):
        self.mod = mod
        self.range = NS(orientations=T, ortho=tuple(w), detector=tuple(p))
        self.shape = (T.shape[0],) + tuple(q.size for q in p)

    def __call__(self, atoms):
        out = np.empty(self.shape, dtype=F64)
        self.mod.RadProj(atoms, self, out)
        return out.view(Sino)

    def L2_derivs(self, atoms, C, order=2):
        res = [self.mod.L2derivs_RadProj(atoms[i], self, C.data, order) for i in range(atoms.size)]
        f = np.vstack([t[0] for t in res])
        df = np.vstack([t[1][None, :] for t in res])
        ddf = np.vstack([t[2][None, :, :] for t in res])
        return (f, df) if order == 1 else (f, df, ddf)


# ---------------------------------------------------------------------------
# problems
# ---------------------------------------------------------------------------
def f32grid(a):
    return np.asarray(a, dtype=np.float32).astype(F64)


def atoms_2d(rng, n, r_lo=2.0, r_hi=4.0, x_half=0.4):
    I = f32grid(rng.uniform(0.5, 1.5, n))
    x = f32grid(rng.uniform(-x_half, x_half, (n, 2)))
    r = f32grid(np.concatenate([rng.uniform(r_lo, r_hi, (n, 2)), rng.normal(0, 0.8, (n, 1))], 1))
    return I, x, r


def atoms_3d(rng, n, r_lo=2.0, r_hi=4.0, x_half=0.35):
    I = f32grid(rng.uniform(0.5, 1.5, n))
    x = f32grid(rng.uniform(-x_half, x_half, (n, 3)))
    r = f32grid(np.concatenate([rng.uniform(r_lo, r_hi, (n, 3)), rng.normal(0, 0.8, (n, 3))], 1))
    return I, x, r


def geom_2d(A, D, half=1.0):
    th = np.linspace(0, np.pi, A, endpoint=False)
    T = f32grid(np.stack([-np.sin(th), np.cos(th)], 1))
    w0 = f32grid(np.stack([np.cos(th), np.sin(th)], 1))
    p0 = f32grid(np.linspace(-half, half, D))
    return T, (w0,), (p0,)


def geom_2p5d(A, D0, D1, half=1.0):
    th = np.linspace(-np.pi / 3, np.pi / 3, A)
    T = f32grid(np.stack([-np.sin(th), np.cos(th)], 1))
    w0 = f32grid(np.stack([np.cos(th), np.sin(th)], 1))
    return T, (w0,), (f32grid(np.linspace(-half, half, D0)), f32grid(np.linspace(-half, half, D1)))


def geom_3d(rng, A, D0, D1, half=1.0):
    # random orthonormal frames (T, w0, w1) as ProjSpace(orientations=, ortho=) takes them
    Q = np.linalg.qr(rng.normal(size=(A, 3, 3)))[0]
    T, w0, w1 = Q[:, :, 0], Q[:, :, 1], Q[:, :, 2]
    return (f32grid(T), (f32grid(w0), f32grid(w1)),
            (f32grid(np.linspace(-half, half, D0)), f32grid(np.linspace(-half, half, D1))))


def put(out, key, **arrs):
    for k, v in arrs.items():
        out["%s_%s" % (key, k)] = np.asarray(v)


# ---------------------------------------------------------------------------
# golden sets
# ---------------------------------------------------------------------------
def pointwise(mods, out):
    rng = np.random.default_rng(101)
    nb2, nb3 = mods["NewtonBases2D"], mods["NewtonBases"]
    rows = []
    for dim, lenT in ((2, 2), (3, 3), (3, 2)):
        for k in range(8):
            if dim == 2:
                I, x, r = atoms_2d(rng, 1)
            else:
                I, x, r = atoms_3d(rng, 1)
            T = rng.normal(size=lenT)
            T /= np.linalg.norm(T)
            y = x[0] + rng.normal(0, 0.12, dim)
            if k == 7:
                # 2 units off the ray through the centre: every output is exactly 0
                Tp = np.pad(T, (0, dim - lenT))
                n = np.array([-Tp[1], Tp[0]]) if dim == 2 else np.cross(Tp, rng.normal(size=3))
                y = x[0] + 2.0 * n / np.linalg.norm(n)
            pr = 3 if dim == 2 else 6
            P = 1 + dim + pr
            Rv = np.zeros(1)
            dR = np.zeros(P)
            ddR = np.zeros((P, P))
            if dim == 2:
                Rf = dev(nb2, "__Rf")(I[0], x[0], r[0], y, T)
                dev(nb2, "__dRf")(I[0], x[0], r[0], y, T, Rv, dR, ddR, 2)
            else:
                Rf = dev(nb3, "__Rf")(I[0], x[0], r[0], y, T)
                dev(nb3, "__dRf_aniso")(I[0], x[0], r[0], y, T, Rv, dR, ddR, 2)
            rows.append(dict(dim=dim, lenT=lenT, I=I[0], x=x[0], r=r[0], y=y, T=T, Rf=Rf,
                             R=Rv[0], dR=dR, ddR=ddR))
    out["pt_n"] = np.array(len(rows))
    for i, row in enumerate(rows):
        put(out, "pt%d" % i, **row)

    # cell maps of the 3D module: y = p0 w0 + p1 w1 (3D) and (p0 w0, p1) (2.5D)
    w0 = rng.normal(size=(3, 3))
    w1 = rng.normal(size=(3, 3))
    Y3 = np.zeros(3)
    dev(nb3, "__tovec3D")(0.3, -0.7, w0, w1, 1, Y3)
    Y25 = np.zeros(3)
    dev(nb3, "__tovec2p5D")(0.3, -0.7, w0[:, :2], w1, 1, Y25)
    put(out, "tovec", w0=w0, w1=w1, y3d=Y3, y2p5d=Y25)


def kernel_set(mods, out, key, modname, dim, gm, T, w, p, I, x, r, iso=False, seed=0):
    """RadProj, L2derivs_RadProj and derivs_RadProj of one module."""
    mod = mods[modname]
    tomo = Tomo(mod, T, w, p)
    atoms = Atoms(dim, iso, I, x, r)
    t0 = time.time()
    R = tomo(atoms).asarray()
    rng = np.random.default_rng(seed)
    # data near the projection, so the L2 residual is not dominated by C
    C = f32grid(R * rng.uniform(0.6, 1.4, R.shape) + rng.normal(0, 0.02, R.shape))
    Csino = C.view(Sino)
    l2 = [mod.L2derivs_RadProj(atoms[j], tomo, Csino.data, 2) for j in range(atoms.size)]
    ip = [mod.derivs_RadProj(atoms[j], tomo, Csino.data, 2) for j in range(atoms.size)]
    put(out, key, gm=gm, I=I, x=x, r=r, T=T, w0=w[0], w1=(w[1] if len(w) > 1 else np.zeros(0)),
        p0=p[0], p1=(p[1] if len(p) > 1 else np.zeros(0)), C=C, R=R,
        l2_f=np.array([np.asarray(t[0]).reshape(()) for t in l2]),
        l2_df=np.stack([t[1] for t in l2]), l2_ddf=np.stack([t[2] for t in l2]),
        ip_f=np.array([np.asarray(t[0]).reshape(()) for t in ip]),
        ip_df=np.stack([t[1] for t in ip]), ip_ddf=np.stack([t[2] for t in ip]))
    print("  %-10s %s: %.1f s" % (key, R.shape, time.time() - t0))


def volproj_set(mods, out, key, modname, dim, I, x, r, n):
    mod = mods[modname]
    y = tuple(f32grid(np.linspace(-0.8, 0.8, n + k)) for k in range(dim))
    u = np.zeros(tuple(v.size for v in y), dtype=F64)
    mod.VolProj(Atoms(dim, False, I, x, r), y, u)
    put(out, key, I=I, x=x, r=r, u=u, **{"y%d" % k: y[k] for k in range(dim)})


def fit_sets(mods, out):
    """NewtonGaussian.linesearch and GD_lib.linesearch_block on one small 2D
    anisotropic L2 problem, run by the reference's own loops on its kernels."""
    nb2 = mods["NewtonBases2D"]
    mgr = mods["manager"]
    loss = mods["transport_loss"].l2_squared_loss(2)
    rng = np.random.default_rng(7)
    T, w, p = geom_2d(12, 28)
    tomo = Tomo(nb2, T, w, p)
    I, x, r = atoms_2d(rng, 4, r_lo=2.5, r_hi=4.0)
    truth = Atoms(2, False, I, x, r)
    data = f32grid(tomo(truth).asarray() + rng.normal(0, 0.01, tomo.shape)).view(Sino)
    I0 = f32grid(I * rng.uniform(0.7, 1.3, I.size))
    x0 = f32grid(x + rng.normal(0, 0.03, x.shape))
    r0 = f32grid(r * rng.uniform(0.85, 1.15, r.shape))
    put(out, "fit", T=T, w0=w[0], p0=p[0], data=data.asarray(), I0=I0, x0=x0, r0=r0)
    reg = mods["regularisation"].null(2)
    with mgr.myManager(device="cpu", fType="float64"):
        t0 = time.time()
        recon = Atoms(2, False, I0, x0, r0)
        rec, E, F = mods["NewtonGaussian"].linesearch(recon, data, [4, 2], loss, reg,
                                                       tomo, view=lambda a: None)
        put(out, "fit_newton", max_iter=np.array([4, 2]), I=rec.I, x=rec.x, r=rec.r, E=E, F=F)
        print("  newton: %d energies, %.1f s" % (E.size, time.time() - t0))
        # linesearch_block takes block t's gradient as df[0], df[1:1+dim], df[1+dim:]
        # by loop position and steps with grad[0] (GD_lib.py:138-151).  With the
        # block string "I" that is the intensity gradient; "xI" shows the slicing
        # (x steps along dF/dI, I along dF/dx0).  "xrI" (the default) raises in
        # the reference for anisotropic atoms: (2,) + (1,3) does not broadcast.
        for blocks, mi in (("I", [3, 1]), ("xI", [2, 1])):
            t0 = time.time()
            recon = Atoms(2, False, I0, x0, r0)
            rec, E, F = mods["GD_lib"].linesearch_block(recon, data, mi, loss, reg, tomo,
                                                         view=lambda a: None, dim=blocks)
            put(out, "fit_gd_" + blocks, max_iter=np.array(mi), I=rec.I, x=rec.x, r=rec.r,
                E=E, F=F)
            print("  gd %s: %d energies, %.1f s" % (blocks, E.size, time.time() - t0))


class SinoS(Sino):
    """A Sino with the ``.space`` (detector, ortho, orientations) that
    KL_GaussRadon.doKL_ProjGDStep_iso reads from its residual."""

    def __array_finalize__(self, obj):
        self.space = getattr(obj, "space", None)


def kl_set(mods, out, root):
    """KL_GaussRadon.doKL_ProjGDStep_iso (KL_GaussRadon.py:57-132), the
    reference's moment-matching atom guess, on a seeded single-atom residual,
    2D anisotropic, with t = 1 and t = 0.5.  Isotropic atoms cannot run: the
    reference's projection of them raises (NewtonBases2D.__to_aniso indexes
    column 1 of an (N, 1) array)."""
    spec = importlib.util.spec_from_file_location("ref_KL_GaussRadon",
                                                  os.path.join(root, "KL_GaussRadon.py"))
    kl = importlib.util.module_from_spec(spec)
    sys.modules["ref_KL_GaussRadon"] = kl
    spec.loader.exec_module(kl)
    nb2, mgr = mods["NewtonBases2D"], mods["manager"]
    rng = np.random.default_rng(23)
    T, w, p = geom_2d(24, 48)
    tomo = Tomo(nb2, T, w, p)
    space = NS(detector=p, ortho=w, orientations=T)
    # the data: one anisotropic atom and small noise (negative cells included)
    I, x, r = atoms_2d(rng, 1, r_lo=2.5, r_hi=3.5, x_half=0.3)
    data = f32grid(tomo(Atoms(2, False, I, x, r)).asarray() +
                   rng.normal(0, 0.01, tomo.shape))
    put(out, "kl", T=T, w0=w[0], p0=p[0], data=data)
    n = 0
    with mgr.myManager(device="cpu", fType="float64"):
        for iso, t in ((False, 1.0), (False, 0.5)):
            t0 = time.time()
            # the atom passed in: its projection is added back to the residual
            # (res = data - R(atom)), so the guess sees the data itself
            a_in = Atoms(2, iso, [0.7], [[0.1, -0.2]], [[3.0]] if iso else [[3.0, 2.5, 0.4]])
            res = (data - tomo(a_in).asarray()).view(SinoS)
            res.space = space
            got = kl.doKL_ProjGDStep_iso(res, a_in, t, tomo)
            put(out, "kl%d" % n, iso=np.array(iso), t=np.array(t), I=got.I, x=got.x, r=got.r)
            print("  KL guess iso=%s t=%.1f: %.1f s" % (iso, t, time.time() - t0))
            n += 1
    out["kl_n"] = np.array(n)


def main(root):
    mods = load_reference(root)
    out = {}
    t0 = time.time()
    pointwise(mods, out)
    rng = np.random.default_rng(11)
    T, w, p = geom_2d(7, 20)
    I, x, r = atoms_2d(rng, 4)
    kernel_set(mods, out, "k2d", "NewtonBases2D", 2, 2, T, w, p, I, x, r, seed=1)
    T, w, p = geom_2p5d(5, 10, 9)
    I, x, r = atoms_3d(rng, 3)
    kernel_set(mods, out, "k2p5d", "NewtonBases", 3, 25, T, w, p, I, x, r, seed=2)
    T, w, p = geom_3d(rng, 5, 10, 9)
    I, x, r = atoms_3d(rng, 3)
    kernel_set(mods, out, "k3d", "NewtonBases", 3, 3, T, w, p, I, x, r, seed=3)
    # pixel-integrated operator (SingleParticleGaussTomo's module)
    T, w, p = geom_2d(6, 14)
    I, x, r = atoms_2d(rng, 3, r_lo=3.0, r_hi=6.0)
    kernel_set(mods, out, "psf2d", "point_spread_functions", 2, 2, T, w, p, I, x, r, seed=4)
    T, w, p = geom_3d(rng, 3, 7, 6)
    I, x, r = atoms_3d(rng, 2, r_lo=3.0, r_hi=6.0)
    kernel_set(mods, out, "psf3d", "point_spread_functions", 3, 3, T, w, p, I, x, r, seed=5)
    # atoms rendered on voxel grids
    I, x, r = atoms_2d(rng, 3)
    volproj_set(mods, out, "vol2d", "NewtonBases2D", 2, I, x, r, 13)
    I, x, r = atoms_3d(rng, 3)
    volproj_set(mods, out, "vol3d", "NewtonBases", 3, I, x, r, 7)
    fit_sets(mods, out)
    kl_set(mods, out, root)
    dst = os.path.join(HERE, "reference_kernels.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, len(out), "arrays in %.0f s" % (time.time() - t0))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
