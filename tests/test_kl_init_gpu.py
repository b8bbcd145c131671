"""Moment-matching atom guess (KL_GaussRadon.doKL_ProjGDStep_iso): the
moment kernel against numpy, the guess against its FP64 oracle, recovery of
a single atom, and greedy insertion in the Newton loop."""
import importlib

import numpy as np
import pytest
import torch

from oracle import gauss_oracle as go
from oracle import kl_init_oracle as ko
from problems import engine_geometry, make_atoms, make_geometry

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"
kl = importlib.import_module(PKG + ".KL_GaussRadon")


@pytest.mark.parametrize("kind", ["2d", "2p5d", "3d"])
def test_moment_kernel_matches_numpy(cuda_ready, kind):
    g = make_geometry(kind, 12, 40, 36)
    rng = np.random.default_rng(1)
    res = rng.normal(size=g.shape).astype(np.float32)
    rr = rng.uniform(size=g.shape).astype(np.float32)
    geom = engine_geometry(g)
    for rrt, t, s in ((None, 1.0, 1.0), (rr, 0.3, 1.7)):
        dev_rr = None if rrt is None else torch.from_numpy(rrt).cuda()
        S0, S1, S2 = kl.sino_moments(geom, torch.from_numpy(res).cuda(), dev_rr, t, s)
        f = np.maximum(0.0, (res if rrt is None else (np.float32(t) * res
                        + np.float32(1 - t) * np.float32(s) * rrt)).astype(np.float64))
        o0, o1, o2 = ko.moments(f, g)
        # FP64 sums of the same FP32 cells; the blend is formed in FP32 on
        # the device (possibly fused), so it may differ in the last bit
        tol = 1e-10 if rrt is None else 1e-6
        for a, b in ((S0, o0), (S1, o1), (S2, o2)):
            assert np.abs(a.cpu().numpy() - b).max() <= tol * max(1.0, np.abs(b).max())


@pytest.mark.parametrize("kind", ["2d", "2p5d", "3d"])
def test_single_atom_is_recovered(cuda_ready, kind):
    g = make_geometry(kind, 30, 96, 96)
    dim = 2 if kind == "2d" else 3
    x = np.array([0.2, -0.1, 0.15][:dim])
    r = np.array([[4.0]])          # standard deviation 1/(sqrt(60) 4)
    data = go.radproj(np.array([1.3]), x.reshape(1, -1), r, g)
    I1, x1, r1 = kl.moment_fit(torch.from_numpy(data).float().cuda(), engine_geometry(g),
                               dim, True)
    assert np.abs(x1 - x).max() < 1e-3
    assert abs(r1[0] - 4.0) < 0.02 * 4.0
    assert abs(I1 - 1.3) < 0.02 * 1.3


@pytest.mark.parametrize("kind,iso", [("2d", True), ("2d", False), ("2p5d", False)])
def test_guess_matches_oracle(cuda_ready, kind, iso):
    g = make_geometry(kind, 24, 64, 60)
    dim = 2 if kind == "2d" else 3
    I, x, r = make_atoms(dim, 3, 7, iso=iso)
    res = go.radproj(I, x, r, g) - 0.3 * go.radproj(I[:1], x[:1], r[:1], g)
    Ie, xe, re = kl.moment_fit(torch.from_numpy(res).float().cuda(), engine_geometry(g),
                               dim, iso, t=0.5)
    Io, xo, ro_ = ko.moment_fit(res.astype(np.float32).astype(np.float64), g, dim, iso, t=0.5)
    assert abs(Ie - Io) <= 1e-3 * abs(Io)
    assert np.abs(xe - xo).max() <= 1e-3 * max(1.0, np.abs(xo).max())
    assert np.abs(re - ro_).max() <= 1e-3 * np.abs(ro_).max()


def test_greedy_insertion_in_newton_loop(cuda_ready):
    sp = importlib.import_module(PKG + ".spaces")
    af = importlib.import_module(PKG + ".atomFuncs")
    fid = importlib.import_module(PKG + ".fidelity")
    regm = importlib.import_module(PKG + ".regularisation")
    sol = importlib.import_module(PKG + ".solvers")
    S = sp.AtomSpace(2, isotropic=True)
    P = sp.ProjSpace(sp.uniform_partition(0, np.pi, 40, nodes_on_bdry=True),
                     sp.uniform_partition(-1.5, 1.5, 128))
    V = sp.VolSpace(sp.uniform_partition([-1, -1], [1, 1], [32, 32]))
    Radon = af.GaussTomo(S, V, P)
    truth = S.element(x=np.array([[0.3, 0.2], [-0.4, -0.1], [0.0, 0.5]]),
                      r=np.array([3.0, 4.0, 3.5]), I=np.array([1.0, 1.5, 0.8]))
    data = Radon(truth)
    recon = S.element(x=np.zeros((3, 2)), r=np.ones(3), I=np.ones(3))
    guess = lambda res, atom: kl.doKL_ProjGDStep_iso(res, atom, 1.0, Radon)
    recon, E, F = sol.Newton_linesearch(recon, data, [3, 1, 5], fid.l2_squared_loss(2),
                                        regm.null(2), Radon, guess=guess)
    # the first guess fits one Gaussian to the whole residual; the sweeps
    # then pull each inserted atom onto a blob
    # (the energy can rise when an atom is inserted, as in the reference)
    assert F[-1] < 0.25 * F[0]
    d = np.linalg.norm(recon.x[:, None, :] - truth.x[None], axis=2).min(axis=0)
    assert d.max() < 0.05
    # far better than the same sweeps from a naive start
    naive = S.element(x=np.zeros((3, 2)), r=np.ones(3), I=np.ones(3))
    _, _, F0 = sol.Newton_linesearch(naive, data, [3, 1], fid.l2_squared_loss(2),
                                     regm.null(2), Radon)
    assert F[-1] < 0.05 * F0[-1]
