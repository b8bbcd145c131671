"""GPU parity of the pixel-integrated (single-particle) operator against the
FP64 oracle restatement of point_spread_functions.py.

Values and gradients: 1e-5 relative (normwise / per parameter entry).
Hessians: 1e-5 relative to each atom's largest Hessian entry; several entries
of the 3D quadrature Hessians are small through cancellation across cells
and carry FP32 rounding of ~1e-5 of their own size (~1e-8 of the matrix)."""
import importlib

import numpy as np
import pytest
import torch

from oracle import gauss_oracle as go
from problems import (atom_normwise_relerr, engine_atoms, engine_geometry, entry_relerr,
                      make_atoms, make_geometry, relerr)

pytestmark = pytest.mark.gpu
TOL = 1e-5
PKG = "2018_dictionary_tomography_gb300"
vol = importlib.import_module(PKG + ".volume")

CASES = {
    "2d": dict(kind="2d", A=12, D0=48, N=10, dim=2),
    "2p5d": dict(kind="2p5d", A=5, D0=24, D1=24, N=5, dim=3),
    "3d": dict(kind="3d", A=4, D0=20, D1=20, N=4, dim=3),
}


def _setup(case, iso=False, seed=0):
    c = CASES[case]
    g = make_geometry(c["kind"], c["A"], c["D0"], c.get("D1"))
    I, x, r = make_atoms(c["dim"], c["N"], seed, iso=iso, rdiag=(3, 6), roff=0.8)
    return g, I, x, r


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("iso", [False, True])
def test_psf_forward_matches_oracle(eng, cuda_ready, case, iso):
    g, I, x, r = _setup(case, iso, seed=51)
    R = eng.radproj(engine_atoms(I, x, r), engine_geometry(g), psf=True).cpu().numpy()
    ref = go.psf_radproj(I, x, r, g)
    assert relerr(R, ref) < TOL


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("mode", ["l2_atom", "inner"])
def test_psf_atom_derivs_match_oracle(eng, cuda_ready, case, mode):
    g, I, x, r = _setup(case, seed=52)
    C = (go.psf_radproj(I[:1] * 1.1, x[:1], r[:1], g) + 0.001).astype(np.float32).astype(np.float64)
    f, gr_, H = eng.atom_derivs(engine_atoms(I, x, r), engine_geometry(g), mode,
                                torch.from_numpy(C).float(), order=2, psf=True)
    kind = "l2" if mode == "l2_atom" else "ip"
    out = [go.psf_atom_derivs(kind, I[j], x[j], r[j], g, C, 2) for j in range(I.size)]
    fo = np.array([o[0] for o in out])
    gro = np.array([o[1] for o in out])
    Ho = np.array([o[2] for o in out])
    assert relerr(f.cpu().numpy(), fo) < TOL
    assert entry_relerr(gr_.cpu().numpy(), gro) < TOL
    assert atom_normwise_relerr(H.cpu().numpy(), Ho) < TOL


def test_psf_iso_derivs_chain_rule(eng, cuda_ready):
    g, I, x, r = _setup("2d", iso=True, seed=53)
    C = go.psf_radproj(I * 0.9, x, r, g).astype(np.float32).astype(np.float64)
    f, gr_, H = eng.atom_derivs(engine_atoms(I, x, r), engine_geometry(g), "l2_atom",
                                torch.from_numpy(C).float(), order=2, psf=True)
    out = [go.psf_atom_derivs("l2", I[j], x[j], r[j], g, C, 2) for j in range(I.size)]
    assert entry_relerr(gr_.cpu().numpy(), np.array([o[1] for o in out])) < TOL
    assert atom_normwise_relerr(H.cpu().numpy(), np.array([o[2] for o in out])) < TOL


def test_psf_fit_fields_give_newton_loop_derivatives(eng, cuda_ready):
    """All-atom field mode = per-atom L2derivs with C = data + R_j - R."""
    g, I, x, r = _setup("2p5d", seed=54)
    data = (go.psf_radproj(I * 1.05, x, r, g) + 0.002).astype(np.float32).astype(np.float64)
    atoms, geom = engine_atoms(I, x, r), engine_geometry(g)
    fw = eng.fit_forward(atoms, geom, torch.from_numpy(data).float(), "l2", psf=True)
    _, gr_, H = eng.atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, 2, psf=True)
    Rt = go.psf_radproj(I, x, r, g)
    assert abs(fw["loss"].item() - go.l2_value(Rt, data)) <= TOL * go.l2_value(Rt, data)
    out = []
    for j in range(I.size):
        Rj = go.psf_radproj(I[j:j + 1], x[j:j + 1], r[j:j + 1], g)
        out.append(go.psf_atom_derivs("l2", I[j], x[j], r[j], g, data + Rj - Rt, 2))
    assert entry_relerr(gr_.cpu().numpy(), np.array([o[1] for o in out])) < TOL
    assert atom_normwise_relerr(H.cpu().numpy(), np.array([o[2] for o in out])) < TOL


@pytest.mark.parametrize("dim", [2, 3])
def test_psf_volproj_matches_oracle(eng, cuda_ready, dim):
    I, x, r = make_atoms(dim, 5, 55, rdiag=(3, 5), roff=0.5)
    n = (24, 20) if dim == 2 else (10, 12, 11)
    coords = [np.linspace(-1, 1, k).astype(np.float32).astype(np.float64) for k in n]
    u = vol.volproj(engine_atoms(I, x, r), coords, psf=True).cpu().numpy()
    ref = go.psf_volproj(I, x, r, coords)
    assert relerr(u, ref) < TOL


def test_single_particle_module_dropin(cuda_ready):
    sp = importlib.import_module(PKG + ".spaces")
    af = importlib.import_module(PKG + ".atomFuncs")
    S = sp.AtomSpace(2, isotropic=False)
    P = sp.ProjSpace(sp.uniform_partition(0, np.pi, 10, True), sp.uniform_partition(-1.5, 1.5, 40))
    V = sp.VolSpace(sp.uniform_partition([-1, -1], [1, 1], [16, 16]))
    Radon = af.SingleParticleGaussTomo(S, V, P)
    I, x, r = make_atoms(2, 4, 56, rdiag=(3, 5))
    atoms = S.element(x, r, I)
    R = Radon(atoms).data
    g = go.Geometry(2, P.orientations, P.ortho[0], P.detector[0])
    assert relerr(R, go.psf_radproj(atoms.I, atoms.x, atoms.r, g)) < TOL
    f, Df, DDf = Radon.L2_derivs(atoms[0], R * 0.9)
    fo, Dfo, DDfo = go.psf_atom_derivs("l2", atoms.I[0], atoms.x[0], atoms.r[0], g, R * 0.9, 2)
    assert relerr(Df[0], Dfo) < TOL
