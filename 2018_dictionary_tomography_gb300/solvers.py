"""Fitting loops on the GPU engine.

``Newton_linesearch`` restates NewtonGaussian.linesearch (NewtonGaussian.py:
18-109) and ``GD_linesearch_block`` restates GD_lib.linesearch_block
(GD_lib.py:82-178): same random sweep order (legacy numpy seed 1), damping and
step-size rules, accept/reject test and break logic, and the same
``(recon, E[:jj], F[:jj])`` return.  The state (sinogram, fit fields, data)
stays in device memory; a step is one derivative call for the moved atom and
one trial of the atom move (gr_atom_step), applied only when accepted --
instead of the reference's three single-atom projections and full-sinogram
host arithmetic per step.

Deviations from the reference, kept deliberately:
* the loops take derivatives of the fidelity they are given (L2 or KL); the
  reference always uses L2 derivatives and uses the fidelity only for the
  accept test;
* GD_linesearch_block slices the gradient of the block it updates and moves
  all of the block's parameters; the reference slices by loop position
  (GD_lib.py:138-143), uses only grad[0] (:151) and crashes for most blocks;
* moment-matching initial guesses (``guess``) and plotting are not provided.

``newton_batched`` is the all-atoms damped Newton loop (one derivative call
for every atom, batched FP64 solves on the device, backtracking on the global
loss) used by the benchmarks and the serving loop.
"""
import numpy as np
import torch

from . import engine


def _max_iter(max_iter):
    if not hasattr(max_iter, "__iter__"):
        return [max_iter, 1]
    max_iter = list(max_iter)
    if len(max_iter) == 1:
        max_iter.append(1)
    return max_iter


def norm(x):
    return float(np.sqrt(np.sum(np.asarray(x, dtype=np.float64) ** 2)))


def _fit_kind(fidelity):
    kind = getattr(fidelity, "kind", "l2")
    bg = float(getattr(fidelity, "background", 0.0))
    return kind, bg


class _DeviceFit:
    """Sinogram, fit fields and data of a fit, resident on the device."""

    def __init__(self, recon, data, fidelity, Radon):
        self.geom = Radon.geometry
        self.dev = self.geom.device
        self.kind, self.bg = _fit_kind(fidelity)
        d = data.asarray() if hasattr(data, "asarray") else data
        self.data = torch.as_tensor(np.asarray(d) if not isinstance(d, torch.Tensor) else d,
                                    dtype=torch.float32).to(self.dev).contiguous()
        self.dim = recon.space.dim
        self.iso = recon.space.isotropic
        self.resync(recon)

    def atoms(self, recon, sl=slice(None)):
        return engine.DeviceAtoms(recon.I[sl], recon.x[sl], recon.r[sl], self.dev)

    def resync(self, recon):
        fw = engine.fit_forward(self.atoms(recon), self.geom, self.data, self.kind,
                                self.bg, want_R=True)
        self.R, self.alpha, self.beta = fw["R"], fw["alpha"], fw["beta"]
        self.loss = float(fw["loss"].item())

    def derivs(self, recon, j, order):
        beta_c = 1.0 if self.kind == "l2" else 0.0
        f, g, H = engine.atom_derivs(self.atoms(recon, slice(j, j + 1)), self.geom, "field",
                                     self.alpha, self.beta, beta_c, order)
        g = g[0].cpu().numpy()
        return g, (H[0].cpu().numpy() if H is not None else None)

    def trial(self, old, new):
        return float(engine.atom_step(old, new, self.geom, self.kind, False, self.R,
                                      self.data, self.alpha, self.beta, self.bg).item())

    def apply(self, old, new):
        engine.atom_step(old, new, self.geom, self.kind, True, self.R, self.data,
                         self.alpha, self.beta, self.bg)


def _single(recon, j, dev, I=None, x=None, r=None):
    return engine.DeviceAtoms(recon.I[j:j + 1] if I is None else I,
                              recon.x[j:j + 1] if x is None else x,
                              recon.r[j:j + 1] if r is None else r, dev)


def step_params(I, x, r, d, dim, iso):
    """The reference's per-atom update with clamps (GD_lib.py:498-522)."""
    I = np.float64(I)
    x = np.asarray(x, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    x_new = x + d[1:dim + 1]
    I_new = max(0.0, I + d[0])
    if iso:
        rr = np.abs(r + d[dim + 1])
    else:
        rr = r + d[dim + 1:]
        if dim == 2:
            if rr[0] < 0:
                rr[0], rr[2] = -rr[0], -rr[2]
            if rr[1] < 0:
                rr[1] = -rr[1]
        else:
            if rr[0] < 0:
                rr[0], rr[3], rr[5] = -rr[0], -rr[3], -rr[5]
            if rr[1] < 0:
                rr[1], rr[4] = -rr[1], -rr[4]
            if rr[2] < 0:
                rr[2] = -rr[2]
    return I_new, x_new, rr


def Newton_linesearch(recon, data, max_iter, fidelity, reg, Radon, view=None,
                      guess=None, tol=1e-4, min_iter=1, resync=True, **kwargs):
    """Damped per-atom Newton sweeps (NewtonGaussian.linesearch).

    With ``guess`` (e.g. ``lambda res, atom: KL_GaussRadon.doKL_ProjGDStep_iso(
    res, atom, 1.0, Radon)``) atoms are inserted one at a time as in the
    reference (NewtonGaussian.py:27-106): atom n is guessed from the residual
    data - R(atoms[:n]) and the first n atoms are swept; with a third entry in
    ``max_iter`` a final round of max_iter[2] sweeps covers all atoms.
    """
    max_iter = _max_iter(max_iter)
    nAtoms = len(recon)
    per = int(np.prod(max_iter[:2]))
    size = per * nAtoms * (nAtoms + 1) // 2 + nAtoms + 2
    if len(max_iter) > 2:
        size += int(max_iter[2]) * int(max_iter[1]) * nAtoms
    E = np.zeros(size if guess is not None else per * nAtoms + 1)
    F = np.zeros_like(E)
    h = [1.0] * nAtoms
    dim, iso = recon.space.dim, recon.space.isotropic
    np.random.seed(1)
    if guess is None:
        st = _DeviceFit(recon, data, fidelity, Radon)
        F[0] = st.loss
        E[0] = F[0] + reg(recon)
        jj = _newton_sweeps(recon, nAtoms, st, h, E, F, 1, max_iter, reg, tol, min_iter,
                            resync, dim, iso)
        return recon, E[:jj], F[:jj]
    d = data.asarray() if hasattr(data, "asarray") else data
    d = np.asarray(d.detach().cpu() if hasattr(d, "detach") else d, dtype=np.float64)
    n = 1
    jj = 1
    while n <= nAtoms + 1:
        if n == nAtoms + 1:
            if len(max_iter) == 2:
                break
            n = nAtoms
            max_iter = [max_iter[2], max_iter[1]]
        else:
            sub = recon[:n].copy()
            res = d - np.asarray(Radon(sub).asarray(), dtype=np.float64)
            recon[n - 1] = guess(res, recon[n - 1].copy())
        sub = recon[:n].copy()
        st = _DeviceFit(sub, data, fidelity, Radon)
        F[jj - 1] = st.loss
        E[jj - 1] = F[jj - 1] + reg(sub)
        jj = _newton_sweeps(sub, n, st, h, E, F, jj, max_iter, reg, tol, min_iter, resync,
                            dim, iso)
        recon[:n] = sub
        n += 1
    return recon, E[:jj], F[:jj]


def _newton_sweeps(recon, n, st, h, E, F, jj, max_iter, reg, tol, min_iter, resync, dim, iso):
    """Sweeps of per-atom damped Newton steps over recon[:n]; returns jj."""
    eps = 1e-4
    for it in range(max_iter[0]):
        BREAK = [True, True]
        for j in np.random.permutation(np.arange(n)):
            for _ in range(max_iter[1]):
                BREAK[1] = True
                df, ddf = st.derivs(recon, j, 2)
                # regulariser terms broadcast as in the reference (:62-66)
                df = df + np.asarray(reg.grad(recon[j]), dtype=np.float64).reshape(-1)
                hr = reg.hess(recon[j])
                ddf = ddf + (hr[0] if np.ndim(hr) == 3 else hr)
                H = 1.0 / h[j]
                for i in range(ddf.shape[0]):
                    ddf[i, i] += H
                dx = np.linalg.solve(ddf, -df)
                I1, x1, r1 = step_params(recon.I[j], recon.x[j], recon.r[j], dx, dim, iso)
                old = _single(recon, j, st.dev)
                new = _single(recon, j, st.dev, np.array([I1]), x1.reshape(1, -1),
                              r1.reshape(1, -1))
                F[jj] = st.loss + st.trial(old, new)
                newrec = recon.copy()
                newrec.I[j], newrec.x[j], newrec.r[j] = I1, x1, r1
                E[jj] = F[jj] + reg(newrec)
                if E[jj] > E[jj - 1]:
                    E[jj] = E[jj - 1]
                    if h[j] > 2 * eps:
                        BREAK[0] = BREAK[1] = False
                    h[j] /= 10
                else:
                    st.apply(old, new)
                    st.loss = F[jj]
                    recon.I[j], recon.x[j], recon.r[j] = I1, x1, r1
                    if norm(dx) > tol:
                        BREAK[0] = BREAK[1] = False
                    h[j] *= 2
                h[j] = min(max(h[j], eps), 1 / eps)
                jj += 1
                if BREAK[1]:
                    break
        if resync:
            st.resync(recon)
        if BREAK[0] and it > min_iter:
            break
    return jj


def GD_linesearch_block(recon, data, max_iter, fidelity, reg, Radon, view=None,
                        dim="xrI", guess=None, tol=1e-4, min_iter=1, resync=True, **kwargs):
    """Per-atom block gradient descent (GD_lib.linesearch_block)."""
    if guess is not None:
        raise NotImplementedError("moment-matching initial guesses are not provided")
    dim = dim.lower()
    blocks = [b for b, c in (("x", "x"), ("r", "r"), ("I", "i")) if c in dim]
    max_iter = _max_iter(max_iter)
    nAtoms = len(recon)
    E = np.zeros(int(np.prod(max_iter[:2])) * nAtoms * len(blocks) + 1)
    F = np.zeros_like(E)
    eps = 1e-8
    h = [[1e-2] * nAtoms for _ in blocks]
    D = recon.space.dim
    st = _DeviceFit(recon, data, fidelity, Radon)
    F[0] = st.loss
    E[0] = F[0] + reg(recon)
    n = nAtoms
    sl = {"I": slice(0, 1), "x": slice(1, 1 + D), "r": slice(1 + D, None)}
    np.random.seed(1)
    jj = 1
    for it in range(max_iter[0]):
        BREAK = [True, True]
        for j in np.random.permutation(np.arange(n)):
            for _ in range(max_iter[1]):
                BREAK[1] = True
                for t, b in enumerate(blocks):
                    df, _h = st.derivs(recon, j, 1)
                    grad = df[sl[b]] + np.asarray(reg.grad(recon[j], axis=b),
                                                  dtype=np.float64).reshape(-1)
                    cur = {"I": np.array([recon.I[j]], dtype=np.float64),
                           "x": recon.x[j].astype(np.float64),
                           "r": recon.r[j].astype(np.float64)}
                    old = cur[b].copy()
                    h[t][j] = min(h[t][j], 1 / max(norm(grad), eps))
                    T = old - h[t][j] * grad
                    new_vals = dict(cur)
                    new_vals[b] = T
                    oldA = _single(recon, j, st.dev)
                    newA = _single(recon, j, st.dev, new_vals["I"], new_vals["x"].reshape(1, -1),
                                   new_vals["r"].reshape(1, -1))
                    F[jj] = st.loss + st.trial(oldA, newA)
                    newrec = recon.copy()
                    newrec.I[j], newrec.x[j], newrec.r[j] = new_vals["I"][0], new_vals["x"], new_vals["r"]
                    E[jj] = F[jj] + reg(newrec)
                    if E[jj] > E[jj - 1]:
                        E[jj] = E[jj - 1]
                        h[t][j] /= 2
                    else:
                        st.apply(oldA, newA)
                        st.loss = F[jj]
                        recon.I[j], recon.x[j], recon.r[j] = new_vals["I"][0], new_vals["x"], new_vals["r"]
                        h[t][j] *= 1.1
                        if norm(old - T) > tol * norm(old):
                            BREAK[0] = BREAK[1] = False
                    h[t][j] = max(h[t][j], eps)
                    jj += 1
                if BREAK[1]:
                    break
        if resync:
            st.resync(recon)
        if BREAK[0] and it > min_iter:
            break
    return recon, E[:jj], F[:jj]


# ---------------------------------------------------------------------------
# all-atoms damped Newton on the device
# ---------------------------------------------------------------------------
def theta_of(I, x, r):
    """(N, P) float64 parameter matrix [I, x, r] on the device."""
    return torch.cat([I.reshape(-1, 1).double(), x.double(), r.reshape(I.numel(), -1).double()], 1).contiguous()


def atoms_of(theta, dim, dev):
    I = theta[:, 0].float().contiguous()
    x = theta[:, 1:1 + dim].float().contiguous()
    r = theta[:, 1 + dim:].float().contiguous()
    return engine.DeviceAtoms(I, x, r, dev)


def newton_batched(atoms, geom, data, iters, fit="l2", background=0.0, lam0=1.0,
                   lam_min=1e-4, lam_max=1e4, max_backtrack=8, tol=0.0, history=None,
                   reg=None):
    """Damped Newton on every atom at once, FP64 Hessian solves on the device.

    Each iteration: one fused forward (fit fields + loss), one derivative call
    (gradient and Hessian of every atom), then backtracking: solve
    (H_j + lam 1) d_j = -g_j for all atoms, re-evaluate the loss, accept when
    it does not increase (lam /= 2), else lam *= 10 and retry.
    With a regulariser (``regularisation.Joubert`` etc.) its per-atom
    gradient and Hessian are added on the device to every block and the
    energy loss + reg(atoms) is what must not increase, as in the
    reference's loop (NewtonGaussian.py:59-66).
    Stops after ``iters`` iterations or when the relative change falls
    below ``tol``.  Returns (DeviceAtoms, energies list).
    """
    use_reg = reg is not None and hasattr(reg, "terms")

    def energy(a, fit_loss):
        if not use_reg:
            return fit_loss
        return fit_loss + float(reg.terms(a, order=1)[0].sum().item())

    dev = geom.device
    dim = atoms.dim
    iso = atoms.iso
    theta = theta_of(atoms.I, atoms.x, atoms.r)
    beta_c = 1.0 if fit == "l2" else 0.0
    fw = engine.fit_forward(atoms, geom, data, fit, background)
    loss = energy(atoms, float(fw["loss"].item()))
    losses = [loss] if history is None else history
    if history is not None:
        history.append(loss)
    lam = torch.full((theta.shape[0],), float(lam0), dtype=torch.float64, device=dev)
    cur = atoms
    rel = float("inf")
    for _ in range(iters):
        _f, g, H = engine.atom_derivs(cur, geom, "field", fw["alpha"], fw["beta"], beta_c, 2)
        if use_reg:
            reg.device_terms(cur, _f, g, H)
        accepted = False
        for _b in range(max_backtrack):
            th_new, _step, _fail = newton_solve_t(dim, iso, g, H, lam, theta)
            trial = atoms_of(th_new, dim, dev)
            fw_new = engine.fit_forward(trial, geom, data, fit, background)
            new_loss = energy(trial, float(fw_new["loss"].item()))
            if new_loss <= loss:
                accepted = True
                rel = (loss - new_loss) / max(abs(loss), 1e-300)
                theta, cur, fw, loss = th_new, trial, fw_new, new_loss
                lam = torch.clamp(lam / 2, lam_min, lam_max)
                break
            lam = torch.clamp(lam * 10, lam_min, lam_max)
        losses.append(loss)
        if not accepted or (tol > 0 and rel < tol):
            break
    return cur, losses


def newton_solve_t(dim, iso, g, H, lam, theta):
    return engine.newton_solve(dim, iso, g.contiguous(), H.contiguous(), lam.contiguous(),
                               theta.contiguous())
