"""GPU tests: torch.autograd wrapper with the hand-written adjoint kernel, and
voxel rendering (VolProj)."""
import importlib

import numpy as np
import pytest
import torch

from oracle import gauss_oracle as go
from problems import (engine_atoms, engine_geometry, entry_relerr, make_atoms,
                      make_geometry, relerr)

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"
ag = importlib.import_module(PKG + ".autograd")
vol = importlib.import_module(PKG + ".volume")


@pytest.mark.parametrize("kind,iso", [("2d", False), ("2p5d", False), ("3d", True)])
def test_autograd_gradient_matches_oracle(cuda_ready, kind, iso):
    g = make_geometry(kind, 9, 40, 36)
    dim = 2 if kind == "2d" else 3
    I, x, r = make_atoms(dim, 7, 41, iso=iso)
    data = (go.radproj(I * 0.9, x + 0.01, r, g)).astype(np.float32).astype(np.float64)
    geom = engine_geometry(g)
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
    It, xt, rt = t(I), t(x), t(r.reshape(len(I), -1))
    R = ag.project(It, xt, rt, geom)
    loss = 0.5 * ((R.double() - torch.from_numpy(data).cuda()) ** 2).sum()
    loss.backward()
    fo, go_, _ = go.all_atom_derivs("l2fit", I, x, r, g, data, 1)
    grad = torch.cat([It.grad.reshape(-1, 1), xt.grad, rt.grad], 1).cpu().numpy()
    assert entry_relerr(grad, go_) < 1e-5


def test_autograd_gradient_central_difference_3d_tilt(cuda_ready):
    """Config-2 style single-axis tilt: central differences with h = 1e-3 of
    the FP64 loss, along random directions scaled per parameter by its natural
    size (I by I, x by the atom width 1/(sqrt(60) r_min), r by r), so that
    h = 1e-3 is a small step for every parameter; the truncation error is
    O(h^2) ~ 1e-6 relative."""
    g = make_geometry("2p5d", 11, 48, 48)
    I, x, r = make_atoms(3, 6, 42, rdiag=(4, 8), roff=1.0)
    data = (go.radproj(I * 1.05, x, r * 0.97, g)).astype(np.float32).astype(np.float64)
    geom = engine_geometry(g)
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda", requires_grad=True)
    It, xt, rt = t(I), t(x), t(r)
    R = ag.project(It, xt, rt, geom)
    (0.5 * ((R.double() - torch.from_numpy(data).cuda()) ** 2).sum()).backward()
    grad = [It.grad.cpu().numpy(), xt.grad.cpu().numpy(), rt.grad.cpu().numpy()]
    rng = np.random.default_rng(43)
    width = 1.0 / (np.sqrt(60.0) * r[:, :3].min(axis=1, keepdims=True))
    scale = [I, np.broadcast_to(width, x.shape), np.maximum(np.abs(r), 1.0)]

    def loss(I_, x_, r_):
        return go.l2_value(go.radproj(I_, x_, r_, g), data)

    h = 1e-3
    for _ in range(4):
        v = [rng.normal(size=a.shape) * s for a, s in zip((I, x, r), scale)]
        fd = (loss(I + h * v[0], x + h * v[1], r + h * v[2]) -
              loss(I - h * v[0], x - h * v[1], r - h * v[2])) / (2 * h)
        an = sum(float(np.sum(a * b)) for a, b in zip(grad, v))
        assert abs(fd - an) <= 1e-4 * abs(an)


def test_autograd_through_torch_optimizer(cuda_ready):
    """A few Adam steps through the autograd wrapper reduce the loss."""
    g = make_geometry("2d", 20, 64)
    I, x, r = make_atoms(2, 5, 44)
    data = torch.from_numpy(go.radproj(I, x, r, g)).float().cuda()
    geom = engine_geometry(g)
    xt = torch.tensor(x + 0.02, dtype=torch.float32, device="cuda", requires_grad=True)
    It = torch.tensor(I, dtype=torch.float32, device="cuda")
    rt = torch.tensor(r, dtype=torch.float32, device="cuda")
    opt = torch.optim.Adam([xt], lr=2e-3)
    losses = []
    for _ in range(20):
        opt.zero_grad()
        L = 0.5 * ((ag.project(It, xt, rt, geom) - data) ** 2).sum()
        L.backward()
        opt.step()
        losses.append(L.item())
    assert losses[-1] < 0.5 * losses[0]


@pytest.mark.parametrize("dim,iso", [(2, True), (2, False), (3, False), (3, True)])
def test_volproj_matches_oracle(eng, cuda_ready, dim, iso):
    I, x, r = make_atoms(dim, 9, 45, iso=iso, rdiag=(2, 4))
    n = (40, 36) if dim == 2 else (20, 18, 22)
    coords = [np.linspace(-1, 1, k).astype(np.float32).astype(np.float64) for k in n]
    u = vol.volproj(engine_atoms(I, x, r), coords).cpu().numpy()
    ref = go.volproj(I, x, r, coords)
    assert u.shape == ref.shape
    assert relerr(u, ref) < 1e-5


def test_gausstomo_discretise(cuda_ready):
    sp = importlib.import_module(PKG + ".spaces")
    af = importlib.import_module(PKG + ".atomFuncs")
    S = sp.AtomSpace(3, isotropic=False)
    V = sp.VolSpace(sp.uniform_partition([-1] * 3, [1] * 3, [16] * 3))
    P = sp.ProjSpace(sp.uniform_partition(0, np.pi, 4, True),
                     sp.uniform_partition([-1, -1], [1, 1], [16, 16]))
    Radon = af.GaussTomo(S, V, P)
    I, x, r = make_atoms(3, 4, 46, rdiag=(2, 4))
    atoms = S.element(x, r, I)
    u = Radon.discretise(atoms).data
    ref = go.volproj(atoms.I, atoms.x, atoms.r, V.coord_vectors)
    assert relerr(u, ref) < 1e-5
