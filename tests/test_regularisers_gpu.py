"""The gr_regulariser kernel against the FP64 oracle (value, gradient,
Hessian per atom), its accumulate mode, the reference-API classes, and a
regularised batched Newton fit."""
import importlib
import os

import numpy as np
import pytest
import torch

from oracle import reg_oracle as ro

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "regularisers.npz"))
PARAMS = {
    "joubert": lambda d: ro.joubert_params(0.7, 0.3, (0.8, 1.3)),
    "mass": lambda d: (0.9, 2.0, 1.5),
    "volume": lambda d: (1.2 ** d, 2.0, 0.5),
    "radius": lambda d: (0.5, 0.8, 2.0),
    "iso": lambda d: (0.6,),
}
SETS = ["d2_aniso", "d2_anisopos", "d2_iso", "d3_aniso", "d3_anisopos", "d3_iso"]
TOL = 1e-10   # FP64 arithmetic on both sides, same float32-grid inputs


def _set(key):
    dim = int(key[1])
    return dim, key.endswith("_iso"), GOLD[key + "_I"], GOLD[key + "_x"], GOLD[key + "_r"]


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


@pytest.mark.parametrize("key", SETS)
@pytest.mark.parametrize("kind", list(PARAMS))
def test_kernel_matches_oracle(eng, cuda_ready, key, kind):
    dim, iso, I, x, r = _set(key)
    p = PARAMS[kind](dim)
    atoms = eng.DeviceAtoms(I, x, r)
    f, g, H = eng.regulariser(kind, p, atoms)
    fo, go, Ho = ro.terms(kind, p, I, x, r, dim, iso)
    f = f.cpu().numpy()
    assert np.array_equal(np.isinf(f), np.isinf(fo))
    fin = np.isfinite(fo)
    assert _rel(f[fin], fo[fin]) < TOL
    assert _rel(g.cpu().numpy(), go) < TOL
    assert _rel(H.cpu().numpy(), Ho) < TOL


def test_accumulate_adds_to_existing_blocks(eng, cuda_ready):
    dim, iso, I, x, r = _set("d3_anisopos")
    atoms = eng.DeviceAtoms(I, x, r)
    P = atoms.n_params()
    rng = np.random.default_rng(0)
    f0 = torch.from_numpy(rng.normal(size=len(I))).cuda()
    g0 = torch.from_numpy(rng.normal(size=(len(I), P))).cuda()
    H0 = torch.from_numpy(rng.normal(size=(len(I), P, P))).cuda()
    f, g, H = f0.clone(), g0.clone(), H0.clone()
    eng.regulariser("radius", PARAMS["radius"](dim), atoms, f, g, H, accumulate=True)
    fo, go, Ho = ro.terms("radius", PARAMS["radius"](dim), I, x, r, dim, iso)
    assert _rel((f - f0).cpu().numpy(), fo) < TOL
    assert _rel((g - g0).cpu().numpy(), go) < TOL
    assert _rel((H - H0).cpu().numpy(), Ho) < TOL


def test_reference_api_classes(cuda_ready):
    regm = importlib.import_module(PKG + ".regularisation")
    sp = importlib.import_module(PKG + ".spaces")
    dim, iso, I, x, r = _set("d2_anisopos")
    S = sp.AtomSpace(2, isotropic=False)
    atoms = S.element(x=x, r=r, I=I)
    reg = regm.Joubert(2, 0.7, 0.3, (0.8, 1.3))
    fo, go, Ho = ro.terms("joubert", PARAMS["joubert"](2), I, x, r, dim, iso)
    assert abs(reg(atoms) - fo.sum()) <= 1e-10 * abs(fo.sum())
    assert _rel(reg.grad(atoms, axis=2), go[:, 3:]) < TOL
    assert _rel(reg.grad(atoms), np.concatenate([go[:, 0], go[:, 1:3].ravel(), go[:, 3:].ravel()])) < TOL
    assert _rel(reg.hess(atoms), Ho) < TOL
    assert abs((2.0 * reg)(atoms) - 2 * fo.sum()) <= 1e-10 * abs(fo.sum())


def test_regularised_batched_newton_decreases_energy(eng, cuda_ready):
    from oracle import gauss_oracle as go
    from problems import engine_geometry, make_atoms, make_geometry
    solvers = importlib.import_module(PKG + ".solvers")
    regm = importlib.import_module(PKG + ".regularisation")
    g = make_geometry("2d", 40, 96)
    I, x, r = make_atoms(2, 12, 5)
    data = torch.from_numpy(go.radproj(I, x, r, g)).float().cuda()
    geom = engine_geometry(g)
    init = eng.DeviceAtoms(I * 1.1, x + 0.01, r)
    reg = regm.Iso(2, 5.0)
    cur, energies = solvers.newton_batched(init, geom, data, 8, reg=reg)
    assert all(b <= a for a, b in zip(energies, energies[1:]))
    # the regulariser pulls the off-diagonal entries towards zero
    off_reg = np.abs(cur.r[:, 2].cpu().numpy()).sum()
    plain_atoms, _ = solvers.newton_batched(eng.DeviceAtoms(I * 1.1, x + 0.01, r), geom, data, 8)
    off_plain = np.abs(plain_atoms.r[:, 2].cpu().numpy()).sum()
    assert off_reg < off_plain
