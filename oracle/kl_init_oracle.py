"""FP64 oracle of the moment-matching atom guess (test infrastructure only).

Restates the iteration of the reference's doKL_ProjGDStep_iso
(KL_GaussRadon.py:57-121) with its moments MOM0/MOM1/MOM2 (:227-253,
:347-368) and orthog_op (:256-343) in numpy, on the oracle's dense FP64
projection, with the same stated differences as the engine's version
(basis-consistent widths r = 1/(sqrt(60) S), off-diagonals 0, start
I = 1, x = 0, S = 0.1).  ``reference_guess`` follows the reference's own
steps and width rule unchanged, so that the golden outputs of its code pin
the shared parts (moments, centre solve, spread, intensity).  Only the tests
use this module.
"""
import numpy as np

from . import gauss_oracle as go


def world_frames(g):
    """T (A, D), detector axes w (K, A, D) and coordinates p (K lists) of an
    oracle geometry; 2.5D tilts embed in 3D with w1 = (0, 0, 1)."""
    if g.gm == 2:
        return g.T, g.w0[None], [g.p0]
    if g.gm == 25:
        z = np.zeros((g.A, 1))
        T = np.concatenate([g.T, z], 1)
        w0 = np.concatenate([g.w0, z], 1)
        w1 = np.tile([[0.0, 0.0, 1.0]], (g.A, 1))
        return T, np.stack([w0, w1]), [g.p0, g.p1]
    return g.T, np.stack([g.w0, g.w1]), [g.p0, g.p1]


def moments(f, g):
    """S0 (A,), S1 (A, K), S2 (A, K) of f >= 0 (A, D0[, D1])."""
    T, w, p = world_frames(g)
    K = len(p)
    S0 = f.reshape(g.A, -1).sum(1)
    S1 = np.zeros((g.A, K))
    S2 = np.zeros((g.A, K))
    if K == 1:
        S1[:, 0] = f @ p[0]
        S2[:, 0] = f @ (p[0] ** 2)
    else:
        S1[:, 0] = np.einsum("ajk,j->a", f, p[0])
        S1[:, 1] = np.einsum("ajk,k->a", f, p[1])
        S2[:, 0] = np.einsum("ajk,j->a", f, p[0] ** 2)
        S2[:, 1] = np.einsum("ajk,k->a", f, p[1] ** 2)
    return S0, S1, S2


def moment_fit(res, g, dim, iso, t=1.0, max_iter=100, rtol=1e-4):
    T, w, p = world_frames(g)
    D, K = T.shape[1], len(p)
    pr = 1 if iso else (3 if dim == 2 else 6)

    def r_of(S):
        r = np.zeros(pr)
        r[:1 if iso else dim] = 1.0 / (np.sqrt(60.0) * S)
        return r

    I, x, S = 1.0, np.zeros(dim), 0.1
    f = np.maximum(0.0, res)
    for _ in range(max_iter):
        S0, S1, S2 = moments(f, g)
        If = S0.sum()
        if If < 1e-8:
            break
        Ify = np.einsum("ka,kad->ad", S1.T, w)
        op = sum(S0[a] * (np.eye(D) - np.outer(T[a], T[a])) for a in range(g.A))
        vec = sum((np.eye(D) - np.outer(T[a], T[a])) @ Ify[a] for a in range(g.A))
        M = np.linalg.solve(op, vec)
        c = np.einsum("kad,d->ak", w, M)
        Ifyy = np.sum(S2 - 2 * c * S1 + c * c * S0[:, None])
        S_new = np.sqrt(max(Ifyy, 0.0) / (K * If))
        x_new = M[:dim]
        RR = go.radproj(np.ones(1), x_new.reshape(1, -1), r_of(S_new).reshape(1, -1), g)
        I_new = If / RR.sum()
        moved = (abs(S - S_new) > rtol * abs(S) or
                 np.linalg.norm(x - x_new) > rtol * np.linalg.norm(x) or
                 abs(I - I_new) > rtol * abs(I))
        I, x, S = I_new, x_new, S_new
        if not moved:
            break
        f = np.maximum(0.0, t * res + (1 - t) * I * RR)
    return I, x, r_of(S)


def reference_guess(res, g, dim, iso, t=1.0):
    """doKL_ProjGDStep_iso (KL_GaussRadon.py:57-132) as the reference runs
    it: ``res`` the data (the residual with this atom's projection added
    back, :68); start I = 1, x = 0, r = 10 on every entry of r[:3] and 0
    after (:82-85); per iteration the moments MOM0/MOM1 (:91, :97, :234-259),
    the centre M from orthog_op (:99-103, :278-346), the centred second
    moment MOM2 about M (:104, :349-394), the spread S = sqrt(Ifyy / ((dim - 1)
    If)) (:109), the width r = S (isotropic) or r[:dim] = 1/S (anisotropic,
    :110-113; the 2D off-diagonal keeps its 10), the intensity from the mass
    of R(atom) (:115-118) and the stop rule on the relative changes of
    (r or 1/r, x, I) (:120-123).  Returns (I, x, r)."""
    T, w, p = world_frames(g)
    D, K = T.shape[1], len(p)
    pr = 1 if iso else (3 if dim == 2 else 6)
    I = 1.0
    x = np.zeros(dim)
    r = np.zeros(pr)
    r[:3] = 10.0
    f = np.maximum(0.0, res)
    for _ in range(100):
        old = [r[0], x.copy(), I]
        if not iso:
            old[0] = 1.0 / old[0]
        If = f.reshape(g.A, -1).sum(1)
        if If.sum() < 1e-8:
            if r[0] < 1e-4:
                return I, x, r
            r = 0.5 * r
            continue
        S0, S1, _S2 = moments(f, g)
        Ify = np.einsum("ka,kad->ad", S1.T, w)
        op = np.zeros((D, D))
        vec = np.zeros(D)
        for a in range(g.A):
            op += If[a] * (np.eye(D) - np.outer(T[a], T[a]))
            vec += Ify[a] - (T[a] @ Ify[a]) * T[a]
        try:
            M = np.linalg.solve(op, vec)
        except np.linalg.LinAlgError:
            M = 0.0 * vec
        c = np.einsum("kad,d->ak", w, M)             # <w_k(a), M>
        if K == 1:
            Ifyy = np.sum(f * (p[0][None, :] - c[:, :1]) ** 2)
        else:
            Ifyy = np.sum(f * ((p[0][None, :, None] - c[:, 0, None, None]) ** 2 +
                               (p[1][None, None, :] - c[:, 1, None, None]) ** 2))
        x = M[:dim].copy()
        S = np.sqrt(Ifyy / ((dim - 1) * If.sum()))
        if iso:
            r[:] = S
        else:
            r[:dim] = 1.0 / S
        RR = go.radproj(np.array([I]), x.reshape(1, -1), r.reshape(1, -1), g)
        A = If.sum() * I / RR.sum()
        RR = RR * (A / I)
        I = A
        if (abs(old[0] - S) > 1e-4 * abs(old[0]) or
                np.linalg.norm(old[1] - M[:dim]) > 1e-4 * np.linalg.norm(old[1]) or
                abs(old[2] - A) > 1e-4 * abs(old[2])):
            f = np.maximum(0.0, t * res + (1 - t) * RR)
        else:
            break
    return I, x, r
