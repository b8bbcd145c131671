"""GPU tests of the drop-in operator API and the fitting loops against the
FP64 oracle restatements."""
import importlib

import numpy as np
import pytest
import torch

from oracle import fit_oracle, gauss_oracle as go
from problems import (engine_atoms, engine_geometry, entry_relerr, make_atoms,
                      make_geometry, relerr)

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"
sp = importlib.import_module(PKG + ".spaces")
af = importlib.import_module(PKG + ".atomFuncs")
fid = importlib.import_module(PKG + ".fidelity")
regm = importlib.import_module(PKG + ".regularisation")
solvers = importlib.import_module(PKG + ".solvers")
NB2 = importlib.import_module(PKG + ".NewtonBases2D")
NB3 = importlib.import_module(PKG + ".NewtonBases")


def _tomo(dim, A, D, iso):
    S = sp.AtomSpace(dim, isotropic=iso)
    if dim == 2:
        P = sp.ProjSpace(sp.uniform_partition(0, np.pi, A, nodes_on_bdry=True),
                         sp.uniform_partition(-1.5, 1.5, D))
    else:
        P = sp.ProjSpace(sp.uniform_partition(-np.pi / 3, np.pi / 3, A, nodes_on_bdry=True),
                         sp.uniform_partition([-1.5, -1.5], [1.5, 1.5], [D, D]))
    V = sp.VolSpace(sp.uniform_partition([-1] * dim, [1] * dim, [16] * dim))
    return S, P, af.GaussTomo(S, V, P)


def _ogeom(P):
    if len(P.detector) == 1:
        return go.Geometry(2, P.orientations, P.ortho[0], P.detector[0])
    return go.Geometry(25, P.orientations, P.ortho[0], P.detector[0], None, P.detector[1])


@pytest.mark.parametrize("dim,iso", [(2, True), (2, False), (3, False)])
def test_gausstomo_call_and_derivs(cuda_ready, dim, iso):
    S, P, Radon = _tomo(dim, 12, 40, iso)
    I, x, r = make_atoms(dim, 6, 31, iso=iso)
    atoms = S.element(x, r, I)
    R = Radon(atoms)
    g = _ogeom(P)
    ref = go.radproj(atoms.I, atoms.x, atoms.r, g)
    assert relerr(R.data, ref) < 1e-5
    C = np.random.default_rng(1).normal(size=P.shape).astype(np.float32)
    f, df, ddf = Radon.derivs(atoms, P.element(C))
    fo, dfo, ddfo = go.all_atom_derivs("ip", atoms.I, atoms.x, atoms.r, g, C, 2)
    assert f.shape == (6, 1) and df.shape == dfo.shape and ddf.shape == ddfo.shape
    assert entry_relerr(df, dfo) < 1e-5 and entry_relerr(ddf, ddfo) < 1e-5
    f2, df2 = Radon.L2_derivs(atoms, C, order=1)
    fo2, dfo2, _ = go.all_atom_derivs("l2", atoms.I, atoms.x, atoms.r, g, C, 1)
    assert relerr(f2.ravel(), fo2) < 1e-5 and entry_relerr(df2, dfo2) < 1e-5


def test_kernel_module_dropin_single_atom(cuda_ready):
    """The four callables with the reference's signatures (NewtonBases2D.py)."""
    S, P, Radon = _tomo(2, 10, 48, False)
    I, x, r = make_atoms(2, 3, 32)
    atoms = S.element(x, r, I)
    R = np.zeros(P.shape, dtype=np.float32)
    NB2.RadProj(atoms, Radon, R)
    g = _ogeom(P)
    assert relerr(R, go.radproj(atoms.I, atoms.x, atoms.r, g)) < 1e-5
    C = R * 0.9
    f, Df, DDf = NB2.L2derivs_RadProj(atoms, Radon, C)
    fo, Dfo, DDfo = go.atom_derivs("l2", atoms.I[0], atoms.x[0], atoms.r[0], g, C, 2)
    assert abs(f - fo) <= 1e-5 * abs(fo)
    assert relerr(Df, Dfo) < 1e-5 and relerr(DDf, DDfo) < 1e-5
    f, Df, DDf = NB2.derivs_RadProj(atoms, Radon, C, order=1)
    fo, Dfo, _ = go.atom_derivs("ip", atoms.I[0], atoms.x[0], atoms.r[0], g, C, 1)
    assert relerr(Df, Dfo) < 1e-5 and DDf.shape == (6, 6)


def test_negative_intensity_forward(eng, cuda_ready):
    g = make_geometry("3d", 6, 32)
    I, x, r = make_atoms(3, 8, 33)
    I[::2] *= -1
    R = eng.radproj(engine_atoms(I, x, r), engine_geometry(g)).cpu().numpy()
    assert relerr(R, go.radproj(I, x, r, g)) < 1e-5
    g2 = make_geometry("2d", 10, 64)
    I2, x2, r2 = make_atoms(2, 8, 34)
    I2[1::2] *= -1
    R2 = eng.radproj(engine_atoms(I2, x2, r2), engine_geometry(g2)).cpu().numpy()
    assert relerr(R2, go.radproj(I2, x2, r2, g2)) < 1e-5


@pytest.mark.parametrize("kind", ["l2", "kl"])
def test_atom_step_trial_and_apply(eng, cuda_ready, kind):
    g = make_geometry("2d", 16, 64)
    I, x, r = make_atoms(2, 5, 35)
    bg = 0.1 if kind == "kl" else 0.0
    rng = np.random.default_rng(3)
    data = go.radproj(I * 1.1, x, r, g) + (bg if kind == "kl" else 0) + rng.uniform(0, 0.02, g.shape)
    data = data.astype(np.float32).astype(np.float64)
    geom = engine_geometry(g)
    dd = torch.from_numpy(data).float().cuda()
    fw = eng.fit_forward(engine_atoms(I, x, r), geom, dd, kind, bg, want_R=True)
    I2, x2, r2 = I.copy(), x.copy(), r.copy()
    x2[2] += 0.03
    r2[2, 0] *= 1.2
    I2[2] *= 0.8
    old = engine_atoms(I[2:3], x[2:3], r[2:3])
    new = engine_atoms(I2[2:3], x2[2:3], r2[2:3])
    dl = eng.atom_step(old, new, geom, kind, False, fw["R"], dd, fw["alpha"], fw["beta"], bg)
    R1 = go.radproj(I, x, r, g)
    R2 = go.radproj(I2, x2, r2, g)
    L = (lambda R: go.l2_value(R, data)) if kind == "l2" else (lambda R: go.kl_value(data, R, bg))
    ref = L(R2) - L(R1)
    assert abs(dl.item() - ref) <= 1e-5 * abs(L(R1))
    eng.atom_step(old, new, geom, kind, True, fw["R"], dd, fw["alpha"], fw["beta"], bg)
    assert relerr(fw["R"].cpu().numpy(), R2) < 1e-5
    fresh = eng.fit_forward(engine_atoms(I2, x2, r2), geom, dd, kind, bg, want_R=True)
    assert relerr(fw["alpha"].cpu().numpy(), fresh["alpha"].cpu().numpy()) < 1e-5


@pytest.mark.parametrize("n", [7, 61])
def test_newton_solve_matches_numpy(eng, cuda_ready, n):
    """Lane groups of P lanes (32 // P atoms a warp, the last lanes idle):
    every atom's damped step equals numpy's, with indefinite blocks (the LU
    fallback) in some warps and partial last warps."""
    rng = np.random.default_rng(4 + n)
    for dim, P, iso in ((2, 6, False), (3, 10, False), (2, 4, True), (3, 5, True)):
        A = rng.normal(size=(n, P, P))
        H = A @ A.transpose(0, 2, 1) + 0.1 * np.eye(P)
        for j in range(3, n, 17):
            H[j] -= 5 * np.eye(P)   # an indefinite block: LU path
        gvec = rng.normal(size=(n, P))
        lam = rng.uniform(0.1, 2, n)
        theta = np.concatenate([rng.uniform(0.5, 1, (n, 1)), rng.normal(size=(n, P - 1))], 1)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        th, step, fail = eng.newton_solve(dim, iso, t(gvec), t(H), t(lam), t(theta))
        for j in range(n):
            d = np.linalg.solve(H[j] + lam[j] * np.eye(P), -gvec[j])
            I1, x1, r1 = solvers.step_params(theta[j, 0], theta[j, 1:1 + dim], theta[j, 1 + dim:],
                                             d, dim, iso)
            want = np.concatenate([[I1], x1, np.atleast_1d(r1)])
            assert np.allclose(th[j].cpu().numpy(), want, rtol=1e-10, atol=1e-12)
            assert np.isclose(step[j].item(), np.linalg.norm(d), rtol=1e-10)
        assert int(fail.sum().item()) == 0


def _fit_problem(kind):
    S, P, Radon = _tomo(2, 20, 64, True)
    I, x, r = make_atoms(2, 4, 36, iso=True, rdiag=(3, 5), box=0.4)
    g = _ogeom(P)
    bg = 0.5 if kind == "kl" else 0.0
    truth = go.radproj(I, x, r, g)
    rng = np.random.default_rng(5)
    if kind == "kl":
        # high counts and a close start keep the KL Hessian blocks positive
        # definite along the path, so FP32 and FP64 runs take the same steps
        data = rng.poisson((truth + bg) * 2000).astype(np.float64) / 2000
        init = (I * rng.uniform(0.9, 1.1, I.size), x + rng.normal(0, 0.01, x.shape), r * 1.05)
    else:
        data = truth + rng.normal(0, 0.01 * truth.max(), truth.shape)
        init = (I * rng.uniform(0.8, 1.2, I.size), x + rng.normal(0, 0.02, x.shape), r * 1.1)
    data = data.astype(np.float32).astype(np.float64)
    init = tuple(a.astype(np.float32).astype(np.float64) for a in init)
    return S, P, Radon, g, data, init, bg


@pytest.mark.parametrize("kind", ["l2", "kl"])
def test_newton_loop_matches_oracle(cuda_ready, kind):
    S, P, Radon, g, data, (I0, x0, r0), bg = _fit_problem(kind)
    recon = S.element(x0, r0, I0)
    fidelity = fid.l2_squared_loss(2) if kind == "l2" else fid.KL_loss(2, bg)
    _, E, F = solvers.Newton_linesearch(recon, P.element(data), [4, 1], fidelity,
                                        regm.null(2), Radon, resync=False)
    (_, _, _), Eo, Fo = fit_oracle.newton(I0, x0, r0, g, data, [4, 1], kind, bg)
    assert E.size == Eo.size
    assert abs(E[-1] - Eo[-1]) <= 1e-4 * abs(Eo[-1])
    assert Eo[-1] < Eo[0]


def test_gd_block_loop_matches_oracle(cuda_ready):
    S, P, Radon, g, data, (I0, x0, r0), bg = _fit_problem("l2")
    recon = S.element(x0, r0, I0)
    _, E, F = solvers.GD_linesearch_block(recon, P.element(data), [3, 1],
                                          fid.l2_squared_loss(2), regm.null(2), Radon,
                                          resync=False)
    (_, _, _), Eo, Fo = fit_oracle.gd_block(I0, x0, r0, g, data, [3, 1])
    assert E.size == Eo.size
    assert abs(E[-1] - Eo[-1]) <= 1e-4 * abs(Eo[-1])


@pytest.mark.parametrize("kind", ["l2", "kl"])
def test_batched_newton_matches_oracle(eng, cuda_ready, kind):
    S, P, Radon, g, data, (I0, x0, r0), bg = _fit_problem(kind)
    geom = engine_geometry(g)
    atoms = engine_atoms(I0, x0, r0)
    dd = torch.from_numpy(data).float().cuda()
    iters = 6 if kind == "l2" else 10
    _, losses = solvers.newton_batched(atoms, geom, dd, iters, kind, bg)
    _, lo = fit_oracle.newton_batched(I0, x0, r0, g, data, iters, kind, bg)
    assert abs(losses[-1] - lo[-1]) <= 1e-4 * abs(lo[-1])
    assert lo[-1] < lo[0]


@pytest.mark.parametrize("case", ["2d_kl", "3d_l2"])
def test_fit_step_graph_matches_direct_calls(eng, cuda_ready, case):
    """engine.FitStep (one graph: H2D, fit, derivatives, D2H) gives exactly
    the results of the direct calls on the same inputs."""
    if case == "2d_kl":
        g = make_geometry("2d", 24, 80)
        I, x, r = make_atoms(2, 12, 41)
        fit, bg, order = "kl", 0.05, 2
    else:
        g = make_geometry("3d", 9, 40, 44)
        I, x, r = make_atoms(3, 10, 42)
        fit, bg, order = "l2", 0.0, 2
    data = go.radproj(I * 1.1, x, r, g) + 0.01
    geom = engine_geometry(g)
    fs = eng.FitStep(geom, len(I), fit=fit, background=bg, order=order)
    loss, gh, Hh = fs.run(I, x, r, data)
    atoms = engine_atoms(I, x, r)
    d = torch.from_numpy(data).float().cuda()
    fw = eng.fit_forward(atoms, geom, d, fit, bg)
    f, gd, Hd = eng.atom_derivs(atoms, geom, "field", fw["alpha"], fw["beta"],
                                1.0 if fit == "l2" else 0.0, order)
    assert loss == fw["loss"].item()
    assert torch.equal(gh, gd.cpu()) and torch.equal(Hh, Hd.cpu())
    # a second run with other atoms reuses the graph
    loss2, gh2, _ = fs.run(I * 0.9, x, r, data)
    atoms2 = engine_atoms(I * 0.9, x, r)
    fw2 = eng.fit_forward(atoms2, geom, d, fit, bg)
    assert loss2 == fw2["loss"].item()
    # angle ranges copied in while the previous range is projected: every
    # cell sums the same atoms in the same order (fields, gradient and
    # Hessian bitwise equal); the loss is a sum of the ranges' losses
    fc = eng.FitStep(geom, len(I), fit=fit, background=bg, order=order, chunks=4)
    assert len(fc.ranges) == 4
    loss_c, gc, Hc = fc.run(I, x, r, data)
    assert torch.equal(gc, gd.cpu()) and torch.equal(Hc, Hd.cpu())
    assert abs(loss_c - fw["loss"].item()) <= 1e-12 * abs(fw["loss"].item())


@pytest.mark.parametrize("accepted", [True, False])
def test_newton_accept_fields_equals_two_launches(eng, cuda_ready, accepted):
    """gr_newton_accept_fields (one launch) leaves every buffer exactly as
    gr_newton_accept followed by gr_accept_fields."""
    rng = np.random.default_rng(8)
    dev = torch.device("cuda")
    n, dim, P = 37, 3, 10

    def state():
        t = lambda a, dt=torch.float64: torch.tensor(a, dtype=dt, device=dev)
        cur = eng.DeviceAtoms(rng.uniform(0.5, 1, n), rng.normal(size=(n, 3)),
                              rng.uniform(5, 9, (n, 6)), dev)
        trial = eng.DeviceAtoms(rng.uniform(0.5, 1, n), rng.normal(size=(n, 3)),
                                rng.uniform(5, 9, (n, 6)), dev)
        return dict(cur=cur, trial=trial, theta=t(rng.normal(size=(n, P))),
                    theta_t=t(rng.normal(size=(n, P))), lam=t(rng.uniform(0.1, 2, n)),
                    loss_cur=t(2.0), loss_trial=t(1.0 if accepted else 3.0),
                    hist=torch.zeros(20, dtype=torch.float64, device=dev),
                    acc=torch.zeros(20, dtype=torch.int32, device=dev),
                    counter=torch.zeros(1, dtype=torch.int32, device=dev),
                    alpha=t(rng.normal(size=(7, 11)), torch.float32),
                    alpha_t=t(rng.normal(size=(7, 11)), torch.float32),
                    beta=t(rng.normal(size=(7, 11)), torch.float32),
                    beta_t=t(rng.normal(size=(7, 11)), torch.float32))

    def clone(s):
        out = {}
        for k, v in s.items():
            if isinstance(v, eng.DeviceAtoms):
                out[k] = eng.DeviceAtoms(v.I.clone(), v.x.clone(), v.r.clone(), dev)
            else:
                out[k] = v.clone()
        return out

    a = state()
    b = clone(a)
    for s, fused in ((a, False), (b, True)):
        eng.newton_accept_into(dim, False, s["loss_cur"], s["loss_trial"], s["theta"],
                               s["theta_t"], s["lam"], 1e-4, 1e4, s["cur"], s["trial"],
                               s["hist"], s["acc"], s["counter"], dev,
                               fields=((s["alpha_t"], s["alpha"], s["beta_t"], s["beta"])
                                       if fused else None))
        if not fused:
            eng.accept_fields_into(s["loss_cur"], s["loss_trial"], s["alpha_t"], s["alpha"],
                                   s["beta_t"], s["beta"], dev)
    for k in a:
        if isinstance(a[k], eng.DeviceAtoms):
            for f in ("I", "x", "r"):
                assert torch.equal(getattr(a[k], f), getattr(b[k], f)), (k, f)
        else:
            assert torch.equal(a[k], b[k]), k
    assert torch.equal(b["alpha"], b["alpha_t"]) == accepted
