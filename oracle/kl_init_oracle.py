"""FP64 oracle of the moment-matching atom guess (test infrastructure only).

Restates the iteration of the reference's doKL_ProjGDStep_iso
(KL_GaussRadon.py:57-121) with its moments MOM0/MOM1/MOM2 (:227-253,
:347-368) and orthog_op (:256-343) in numpy, on the oracle's dense FP64
projection, with the same stated differences as the engine's version
(basis-consistent widths r = 1/(sqrt(60) S), off-diagonals 0, start
I = 1, x = 0, S = 0.1).  Only the tests use it.
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
