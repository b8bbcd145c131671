"""The CUDA engine, through the drop-in kernel modules and fitting loops,
against outputs of the reference's own code.

The golden file holds what the reference's NewtonBases2D / NewtonBases /
point_spread_functions callables and its NewtonGaussian / GD_lib loops
returned on seeded inputs (run in FP64 through the numba stand-in,
``tests/golden/make_ref_golden.py``).  Our modules are called exactly as the
reference's GaussTomo calls its own (GaussDictCode/atomFuncs.py:115-158) and
must agree within the FP32 bar: 1e-5 relative (arrays normwise; gradients and
Hessians per atom, scaled by the largest entry of that atom's array).  Fits:
the same energy after the same number of steps, within 1e-4 relative.
"""
import importlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                    "reference_kernels.npz")
TOL = 1e-5


class NS:
    def __init__(self, **kw):
        self.__dict__.update(kw)


@pytest.fixture(scope="module")
def z():
    return np.load(GOLD)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


def _module(key):
    name = {"k2d": "NewtonBases2D", "k2p5d": "NewtonBases", "k3d": "NewtonBases",
            "psf2d": "point_spread_functions", "psf3d": "point_spread_functions",
            "vol2d": "NewtonBases2D", "vol3d": "NewtonBases"}[key]
    return importlib.import_module(PKG + "." + name)


def _rad(z, key):
    g = lambda k: z["%s_%s" % (key, k)]
    ortho = (g("w0"),) if g("w1").size == 0 else (g("w0"), g("w1"))
    det = (g("p0"),) if g("p1").size == 0 else (g("p0"), g("p1"))
    return NS(range=NS(orientations=g("T"), ortho=ortho, detector=det))


def _atoms(I, x, r):
    return NS(I=np.asarray(I), x=np.asarray(x), r=np.asarray(r),
              space=NS(isotropic=False, dim=np.asarray(x).shape[-1]))


@pytest.mark.parametrize("key", ["k2d", "k2p5d", "k3d", "psf2d", "psf3d"])
def test_dropin_callables_match_reference(cuda_ready, z, key):
    g = lambda k: z["%s_%s" % (key, k)]
    mod, Rad = _module(key), _rad(z, key)
    R = np.zeros(g("R").shape, dtype=np.float32)
    mod.RadProj(_atoms(g("I"), g("x"), g("r")), Rad, R)
    assert rel(R, g("R")) < TOL
    for kind, fn in (("l2", mod.L2derivs_RadProj), ("ip", mod.derivs_RadProj)):
        for j in range(g("I").size):
            a = _atoms(g("I")[j:j + 1], g("x")[j:j + 1], g("r")[j:j + 1])
            f, df, ddf = fn(a, Rad, g("C"), 2)
            assert abs(f - g(kind + "_f")[j]) <= TOL * max(abs(g(kind + "_f")[j]), 1e-30) \
                or rel(f, g(kind + "_f")[j]) < TOL
            assert rel(df, g(kind + "_df")[j]) < TOL
            assert rel(ddf, g(kind + "_ddf")[j]) < TOL


@pytest.mark.parametrize("key", ["vol2d", "vol3d"])
def test_dropin_volproj_matches_reference(cuda_ready, z, key):
    g = lambda k: z["%s_%s" % (key, k)]
    dim = g("x").shape[1]
    y = tuple(g("y%d" % k) for k in range(dim))
    u = np.zeros(g("u").shape, dtype=np.float32)
    _module(key).VolProj(_atoms(g("I"), g("x"), g("r")), y, u)
    assert rel(u, g("u")) < TOL


def _fit_setup(z):
    sp = importlib.import_module(PKG + ".spaces")
    af = importlib.import_module(PKG + ".atomFuncs")
    S = sp.AtomSpace(2, isotropic=False)
    P = sp.ProjSpace(orientations=z["fit_T"], ortho=(z["fit_w0"],), detector=(z["fit_p0"],))
    V = sp.VolSpace(sp.uniform_partition([-1, -1], [1, 1], [16, 16]))
    return S, P, af.GaussTomo(S, V, P)


def test_newton_linesearch_matches_reference_loop(cuda_ready, z):
    """solvers.Newton_linesearch against NewtonGaussian.linesearch run by the
    reference on its own kernels: same number of steps, same energies."""
    fid = importlib.import_module(PKG + ".fidelity")
    regm = importlib.import_module(PKG + ".regularisation")
    solvers = importlib.import_module(PKG + ".solvers")
    S, P, Radon = _fit_setup(z)
    recon = S.element(z["fit_x0"], z["fit_r0"], z["fit_I0"])
    _, E, _F = solvers.Newton_linesearch(recon, P.element(z["fit_data"]),
                                         list(z["fit_newton_max_iter"]), fid.l2_squared_loss(2),
                                         regm.null(2), Radon)
    Er = z["fit_newton_E"]
    assert E.size == Er.size
    assert np.all(np.abs(E - Er) <= 1e-4 * np.abs(Er))


def test_gd_linesearch_block_matches_reference_loop(cuda_ready, z):
    """solvers.GD_linesearch_block on intensities (the block string for which
    the reference's position-sliced gradient is the block's own)."""
    fid = importlib.import_module(PKG + ".fidelity")
    regm = importlib.import_module(PKG + ".regularisation")
    solvers = importlib.import_module(PKG + ".solvers")
    S, P, Radon = _fit_setup(z)
    recon = S.element(z["fit_x0"], z["fit_r0"], z["fit_I0"])
    _, E, _F = solvers.GD_linesearch_block(recon, P.element(z["fit_data"]),
                                           list(z["fit_gd_I_max_iter"]), fid.l2_squared_loss(2),
                                           regm.null(2), Radon, dim="I")
    Er = z["fit_gd_I_E"]
    assert E.size == Er.size
    assert np.all(np.abs(E - Er) <= 1e-4 * np.abs(Er))
