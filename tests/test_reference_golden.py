"""The FP64 oracle against outputs of the reference's own code.

``tests/golden/reference_kernels.npz`` holds outputs of the reference's Numba
kernel modules and fitting loops, executed on the CPU through a numba stand-in
that emulates the CUDA launch in FP64 (``tests/golden/make_ref_golden.py``,
``tests/golden/ref_numba_stub.py``).  Every oracle routine the parity tests
rely on must reproduce them to 1e-12 relative (the two sides differ only in
FP64 rounding order).  No GPU.
"""
import os

import numpy as np
import pytest

from oracle import fit_oracle
from oracle import gauss_oracle as go

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                    "reference_kernels.npz")
TOL = 1e-12


@pytest.fixture(scope="module")
def z():
    return np.load(GOLD)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


def geometry(z, key):
    g = lambda k: z["%s_%s" % (key, k)]
    w1 = g("w1") if g("w1").size else None
    p1 = g("p1") if g("p1").size else None
    return go.Geometry(int(g("gm")), g("T"), g("w0"), g("p0"), w1, p1)


def test_pointwise_cell_derivatives_match_reference(z):
    """__Rf/__dRf (NewtonBases2D.py:39-243) and __Rf/__dRf_aniso
    (NewtonBases.py:262-528), 3D and 2.5D ray directions, one cell off the
    support (all zeros)."""
    n = int(z["pt_n"])
    assert n >= 24
    for i in range(n):
        g = lambda k: z["pt%d_%s" % (i, k)]
        R, dR, ddR = go.point_derivs(int(g("dim")), int(g("lenT")), g("I"), g("x"), g("r"),
                                     g("y"), g("T"), 2)
        assert rel(R, g("R")) <= TOL
        assert rel(R, g("Rf")) <= TOL
        assert rel(dR, g("dR")) <= TOL
        assert rel(ddR, g("ddR")) <= TOL
        if i % 8 == 7:
            assert g("R") == 0 and not np.any(g("dR")) and not np.any(g("ddR"))


def test_cell_maps_match_reference(z):
    """__tovec3D / __tovec2p5D (NewtonBases.py:677-688): the cell centre as
    the oracle's Geometry builds it."""
    w0, w1 = z["tovec_w0"], z["tovec_w1"]
    p0, p1, a = 0.3, -0.7, 1
    assert rel(p0 * w0[a] + p1 * w1[a], z["tovec_y3d"]) <= TOL
    y25 = np.array([p0 * w0[a, 0], p0 * w0[a, 1], p1])
    assert rel(y25, z["tovec_y2p5d"]) <= TOL


@pytest.mark.parametrize("key", ["k2d", "k2p5d", "k3d", "psf2d", "psf3d"])
def test_module_callables_match_reference(z, key):
    """RadProj, L2derivs_RadProj and derivs_RadProj (order 2) of
    NewtonBases2D / NewtonBases / point_spread_functions, per atom."""
    g = lambda k: z["%s_%s" % (key, k)]
    geom = geometry(z, key)
    psf = key.startswith("psf")
    R = (go.psf_radproj if psf else go.radproj)(g("I"), g("x"), g("r"), geom)
    assert np.abs(g("R")).max() > 0
    assert rel(R, g("R")) <= TOL
    derivs = go.psf_atom_derivs if psf else go.atom_derivs
    for kind in ("l2", "ip"):
        for j in range(g("I").size):
            f, df, ddf = derivs(kind, g("I")[j], g("x")[j], g("r")[j], geom, g("C"), 2)
            assert rel(f, g(kind + "_f")[j]) <= TOL
            assert rel(df, g(kind + "_df")[j]) <= TOL
            assert rel(ddf, g(kind + "_ddf")[j]) <= TOL


@pytest.mark.parametrize("key", ["vol2d", "vol3d"])
def test_volproj_matches_reference(z, key):
    g = lambda k: z["%s_%s" % (key, k)]
    dim = g("x").shape[1]
    u = go.volproj(g("I"), g("x"), g("r"), [g("y%d" % k) for k in range(dim)])
    assert np.abs(g("u")).max() > 0
    assert rel(u, g("u")) <= TOL


def _fit_geom(z):
    return go.Geometry(2, z["fit_T"], z["fit_w0"], z["fit_p0"])


def test_newton_fit_oracle_matches_reference_loop(z):
    """NewtonGaussian.linesearch (NewtonGaussian.py:18-109) run by the
    reference on its own kernels: same energy history and final atoms."""
    (I, x, r), E, F = fit_oracle.newton(z["fit_I0"], z["fit_x0"], z["fit_r0"], _fit_geom(z),
                                        z["fit_data"], list(z["fit_newton_max_iter"]))
    assert E.size == z["fit_newton_E"].size
    assert rel(E, z["fit_newton_E"]) <= TOL
    assert rel(F, z["fit_newton_F"]) <= TOL
    for a, k in ((I, "I"), (x, "x"), (r, "r")):
        assert rel(a, z["fit_newton_" + k]) <= 1e-10
    assert E[-1] < E[0]


@pytest.mark.parametrize("blocks,slicing", [("I", "block"), ("I", "reference"),
                                            ("xI", "reference")])
def test_gd_block_fit_oracle_matches_reference_loop(z, blocks, slicing):
    """GD_lib.linesearch_block (GD_lib.py:82-178).  For the block string "I"
    the reference's position-sliced gradient is the intensity gradient, so
    the corrected rule agrees with it; for "xI" only the oracle's
    reference-slicing mode does (x moves along dF/dI, I along dF/dx0)."""
    key = "fit_gd_" + blocks
    (I, x, r), E, F = fit_oracle.gd_block(z["fit_I0"], z["fit_x0"], z["fit_r0"], _fit_geom(z),
                                          z["fit_data"], list(z[key + "_max_iter"]),
                                          dim_str=blocks, slicing=slicing)
    assert E.size == z[key + "_E"].size
    assert rel(E, z[key + "_E"]) <= TOL
    for a, k in ((I, "I"), (x, "x"), (r, "r")):
        assert rel(a, z[key + "_" + k]) <= 1e-10


def test_gd_block_corrected_rule_departs_from_reference_slicing(z):
    """The deviation is real: with blocks "xI" the corrected rule does not
    follow the reference's trajectory."""
    key = "fit_gd_xI"
    _, E, _ = fit_oracle.gd_block(z["fit_I0"], z["fit_x0"], z["fit_r0"], _fit_geom(z),
                                  z["fit_data"], list(z[key + "_max_iter"]), dim_str="xI")
    n = min(E.size, z[key + "_E"].size)
    assert rel(E[:n], z[key + "_E"][:n]) > 1e-8


def _kl_geom(z):
    return go.Geometry(2, z["kl_T"], z["kl_w0"], z["kl_p0"])


def test_kl_guess_oracle_matches_reference(z):
    """KL_GaussRadon.doKL_ProjGDStep_iso (KL_GaussRadon.py:57-132) run by the
    reference: the oracle's restatement of its rule gives the same atom."""
    from oracle import kl_init_oracle as ko
    assert int(z["kl_n"]) >= 2
    for i in range(int(z["kl_n"])):
        g = lambda k: z["kl%d_%s" % (i, k)]
        I, x, r = ko.reference_guess(z["kl_data"], _kl_geom(z), 2, bool(g("iso")), float(g("t")))
        assert rel(I, g("I")[0]) <= TOL
        assert rel(x, g("x")[0]) <= TOL
        assert rel(r, g("r")[0]) <= TOL


def test_kl_guess_departs_only_in_width_rule(z):
    """Where the engine's guess departs from the reference's, on the t = 1
    golden (the blend weight that makes the moments those of the data): the
    centre and the spread S are the reference's; the widths follow the
    kernels' basis, r = 1/(sqrt(60) S) instead of 1/S, with the 2D
    off-diagonal 0 instead of the start value 10 the reference leaves; the
    intensity, matched to the mass of R(atom), follows the widths."""
    from oracle import kl_init_oracle as ko
    i = [k for k in range(int(z["kl_n"])) if float(z["kl%d_t" % k]) == 1.0][0]
    g = lambda k: z["kl%d_%s" % (i, k)]
    I, x, r = ko.moment_fit(z["kl_data"], _kl_geom(z), 2, False, 1.0)
    assert rel(x, g("x")[0]) <= TOL
    assert rel(np.sqrt(60.0) * r[:2], g("r")[0][:2]) <= TOL
    assert r[2] == 0.0 and g("r")[0][2] == 10.0
    assert rel(I, g("I")[0]) > 0.5
