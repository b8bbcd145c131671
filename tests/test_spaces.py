"""CPU tests of the ODL-free dictionary spaces (GaussDictCode/dictionary_def.py)
and geometry helpers (GaussDictCode/atomFuncs.py:13-74)."""
import importlib

import numpy as np
import pytest

from oracle import gauss_oracle as go

sp = importlib.import_module("2018_dictionary_tomography_gb300.spaces")
geo = importlib.import_module("2018_dictionary_tomography_gb300.geometry")


def test_theta_to_vec_and_perp_match_oracle_restatement():
    th = [np.linspace(0, np.pi, 7)]
    assert np.allclose(geo.theta_to_vec(th), go.theta_to_vec(th))
    assert np.allclose(geo.perp(th)[0], go.perp(th)[0])
    th3 = [np.linspace(0, 1, 3), np.linspace(-1, 1, 4)]
    assert np.allclose(geo.theta_to_vec(th3), go.theta_to_vec(th3))
    for a, b in zip(geo.perp(th3), go.perp(th3)):
        assert np.allclose(a, b)
    # orthonormal frames
    T = geo.theta_to_vec(th3).reshape(-1, 3)
    w0, w1 = [w.reshape(-1, 3) for w in geo.perp(th3)]
    for u, v in ((T, w0), (T, w1), (w0, w1)):
        assert np.allclose(np.sum(u * v, 1), 0)


def test_atom_element_layouts_follow_reference():
    S = sp.AtomSpace(2, isotropic=False)
    a = S.element([[.1, .2], [.3, .4]], [1.5, 2.5], 1.0)
    assert a.x.shape == (2, 2) and a.r.shape == (2, 3) and a.I.shape == (2,)
    assert np.allclose(a.r, [[1.5, 1.5, 0], [2.5, 2.5, 0]])
    b = sp.AtomSpace(3, isotropic=True).random(5, seed=1)
    assert b.r.shape == (5, 1) and b.x.shape == (5, 3) and len(b) == 5
    c = b[2]
    assert c.x.shape == (1, 3) and c.r.shape == (1, 1)
    b[2] = b[3]
    assert np.allclose(b.x[2], b.x[3])
    with pytest.raises(ValueError):
        sp.AtomElement(sp.AtomSpace(2, False), np.zeros((2, 2)), np.ones((2, 2)), 1)
    d = S.element(np.concatenate([a.I[:, None], a.x, a.r], 1))
    assert np.allclose(d.x, a.x) and np.allclose(d.r, a.r)


def test_proj_space_from_partitions():
    ang = sp.uniform_partition(0, np.pi, 30, nodes_on_bdry=True)
    det = sp.uniform_partition(-1.5, 1.5, 64)
    P = sp.ProjSpace(ang, det)
    assert P.shape == [30, 64]
    assert P.orientations.shape == (30, 2) and len(P.ortho) == 1
    assert np.isclose(P.detector[0][1] - P.detector[0][0], 3 / 64)
    e = P.element(np.ones(P.shape))
    assert np.allclose((e - e * 2).data, -1)
    with pytest.raises(ValueError):
        P.element(np.ones((3, 3)))
    P3 = sp.ProjSpace(sp.uniform_partition([0, 0], [np.pi, 1], [4, 3]),
                      sp.uniform_partition([-1, -1], [1, 1], [16, 16]))
    assert P3.shape == [12, 16, 16] and len(P3.ortho) == 2


def test_frame_records_dual_rows():
    rng = np.random.default_rng(0)
    T = rng.normal(size=(5, 3))
    w0 = rng.normal(size=(5, 3))
    w1 = rng.normal(size=(5, 3))
    rec, kdet = geo.frame_records(T, (w0, w1), 2)
    assert kdet == 2 and rec.shape == (5, 24)
    B = np.stack([w0, w1, T], 2).astype(np.float32).astype(np.float64)
    inv = np.linalg.inv(B)
    assert np.allclose(rec[:, 9:12], inv[:, 0, :], rtol=1e-5, atol=1e-5)
    # hi + lo carries the FP64 dual rows to ~1e-14 (the kernels' centre B^-1 x)
    for k in range(2):
        full = rec[:, 9 + 3 * k:12 + 3 * k].astype(np.float64) + rec[:, 15 + 3 * k:18 + 3 * k]
        assert np.abs(full - inv[:, k, :]).max() <= 1e-13 * np.abs(inv).max()
    rec2, kdet2 = geo.frame_records(T[:, :2], (w0[:, :2],), 1)
    B2 = np.stack([w0[:, :2], T[:, :2]], 2).astype(np.float32).astype(np.float64)
    inv2 = np.linalg.inv(B2)
    assert kdet2 == 1 and rec2.shape == (5, 8)
    full2 = rec2[:, 4:6].astype(np.float64) + rec2[:, 6:8]
    assert np.abs(full2 - inv2[:, 0, :]).max() <= 1e-13 * np.abs(inv2).max()
    with pytest.raises(ValueError):
        geo.uniform_grid([0.0, 1.0, 3.0])
    with pytest.raises(ValueError):
        geo.uniform_grid([1.0, 0.0, -1.0])


def test_gausstomo_refuses_cpu_like_reference():
    at = importlib.import_module("2018_dictionary_tomography_gb300.atomFuncs")
    S = sp.AtomSpace(2)
    P = sp.ProjSpace(sp.uniform_partition(0, np.pi, 4, True), sp.uniform_partition(-1, 1, 8))
    with pytest.raises(ValueError):
        at.GaussTomo(S, None, P, device="cpu")
