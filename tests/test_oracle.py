"""CPU checks of the oracle itself (known answers, finite differences,
internal consistency).  No GPU."""
import os

import numpy as np
import pytest

from oracle import gauss_oracle as go
from problems import make_atoms, make_geometry, relerr

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pointwise.npz")


def test_oracle_matches_sympy_known_answers():
    """Per-cell value/gradient/Hessian of 1/2(R - C)^2 against the reference's
    sympy self-test expression regenerated with the kernels' basis
    (tests/golden/make_golden.py)."""
    z = np.load(GOLD)
    n = int(z["n"])
    assert n >= 10
    for i in range(n):
        g = lambda k: z["c%d_%s" % (i, k)]
        dim, lenT = int(g("dim")), int(g("lenT"))
        R, dR, ddR = go.point_derivs(dim, lenT, g("I"), g("x"), g("r"), g("y"),
                                     g("T")[:lenT], 2)
        C = float(g("C"))
        F = 0.5 * (R - C) ** 2
        dF = (R - C) * dR
        ddF = np.outer(dR, dR) + (R - C) * ddR
        assert abs(R - g("R")) <= 1e-12 * abs(g("R"))
        assert abs(F - g("F")) <= 1e-12 * max(abs(g("F")), 1e-300)
        assert relerr(dF, g("dF")) < 1e-12
        assert relerr(ddF, g("ddF")) < 1e-12


@pytest.mark.parametrize("dim,lenT", [(2, 2), (3, 3), (3, 2)])
def test_oracle_point_derivs_finite_difference(dim, lenT):
    rng = np.random.default_rng(3)
    pr = 3 if dim == 2 else 6
    I = 1.3
    x = rng.uniform(-0.2, 0.2, dim)
    r = np.concatenate([rng.uniform(2, 4, dim), rng.normal(0, 0.5, pr - dim)])
    T = rng.normal(size=lenT)
    T /= np.linalg.norm(T)
    y = x + rng.normal(0, 0.08, dim)
    th = np.concatenate([[I], x, r])

    def val(t):
        return go.point_derivs(dim, lenT, t[0], t[1:1 + dim], t[1 + dim:], y, T, 1)[0]

    R, dR, ddR = go.point_derivs(dim, lenT, I, x, r, y, T, 2)
    h = 1e-5
    fd = np.zeros_like(dR)
    fdd = np.zeros_like(ddR)
    for i in range(th.size):
        e = np.zeros_like(th)
        e[i] = h
        fd[i] = (val(th + e) - val(th - e)) / (2 * h)
        gp = go.point_derivs(dim, lenT, *(lambda t: (t[0], t[1:1 + dim], t[1 + dim:]))(th + e), y, T, 1)[1]
        gm = go.point_derivs(dim, lenT, *(lambda t: (t[0], t[1:1 + dim], t[1 + dim:]))(th - e), y, T, 1)[1]
        fdd[i] = (gp - gm) / (2 * h)
    assert relerr(dR, fd) < 1e-7
    assert relerr(ddR, fdd) < 1e-6


def test_oracle_field_kind_equals_l2fit():
    """The all-atoms L2 derivatives (Newton-loop semantics) equal the weight
    field form with alpha = R - data, beta = 1."""
    g = make_geometry("2d", 9, 48)
    I, x, r = make_atoms(2, 3, 1)
    rng = np.random.default_rng(2)
    data = rng.normal(size=g.shape) * 0.1
    a = go.all_atom_derivs("l2fit", I, x, r, g, data, 2)
    Rt = go.radproj(I, x, r, g)
    b = go.all_atom_derivs("field", I, x, r, g, Rt - data, 2, beta=np.ones(g.shape))
    assert relerr(b[1], a[1]) < 1e-12
    assert relerr(b[2], a[2]) < 1e-12


def test_oracle_iso_equals_aniso_chain_rule():
    g = make_geometry("3d", 6, 24)
    I, x, r = make_atoms(3, 2, 4, iso=True)
    ra = go.to_aniso(r, 3)
    C = np.random.default_rng(5).normal(size=g.shape)
    fi, gi, Hi = go.all_atom_derivs("ip", I, x, r, g, C, 2)
    fa, ga, Ha = go.all_atom_derivs("ip", I, x, ra, g, C, 2)
    gc, Hc = go.collapse_iso(ga, Ha, 3)
    assert relerr(gi, gc) < 1e-14 and relerr(Hi, Hc) < 1e-14
    R1 = go.radproj(I, x, r, g)
    R2 = go.radproj(I, x, ra, g)
    assert relerr(R1, R2) == 0.0


def test_oracle_f32_twin_close_to_f64():
    g = make_geometry("2d", 20, 64)
    I, x, r = make_atoms(2, 16, 6)
    R64 = go.radproj(I, x, r, g)
    R32 = go.radproj(I, x, r, g, dtype=np.float32)
    assert relerr(R32, R64) < 1e-5


def test_oracle_thread_count_invariance():
    g = make_geometry("2d", 12, 40)
    I, x, r = make_atoms(2, 4, 7)
    C = np.random.default_rng(8).normal(size=g.shape)
    a = go.all_atom_derivs("ip", I, x, r, g, C, 2, nthreads=1)
    b = go.all_atom_derivs("ip", I, x, r, g, C, 2, nthreads=4)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("kind,dim,args", [("2d", 2, (30, 96)), ("2p5d", 3, (9, 40, 36)),
                                           ("3d", 3, (9, 40, 44))])
def test_boxed_evaluation_equals_dense(kind, dim, args):
    """The shadow-box projection and per-atom derivatives visit only the
    cells an atom can reach and give the dense results (projection bitwise)."""
    g = make_geometry(kind, *args)
    I, x, r = make_atoms(dim, 30, 3)
    assert np.array_equal(go.radproj(I, x, r, g), go.radproj_boxed(I, x, r, g))
    C = np.random.default_rng(5).normal(size=g.shape)
    B = np.random.default_rng(6).uniform(0.5, 2, size=g.shape)
    for j in range(0, 30, 7):
        for k, beta in (("ip", None), ("field", B)):
            a = go.atom_derivs(k, I[j], x[j], r[j], g, C, 2, beta=beta)
            b = go.atom_derivs(k, I[j], x[j], r[j], g, C, 2, beta=beta, boxed=True)
            assert abs(a[0] - b[0]) <= 1e-13 * max(abs(a[0]), 1e-300)
            assert relerr(b[1], a[1]) < 1e-13 and relerr(b[2], a[2]) < 1e-13
