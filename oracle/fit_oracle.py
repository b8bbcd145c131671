"""FP64 restatement of the reference's fitting loops (test infrastructure).

Newton: NewtonGaussian.linesearch (NewtonGaussian.py:18-109) with the step of
GD_lib._step (GD_lib.py:492-536).  GD: GD_lib.linesearch_block
(GD_lib.py:82-178) with the gradient of the updated block (the reference's
slicing by loop position and use of grad[0] are treated as defects, see the
product's solvers module).  Derivatives come from the fidelity in use: L2
(the reference's L2derivs_RadProj) or KL (weight fields 1 - f/g, f/g^2).
Projections and per-atom derivatives visit each atom's shadow box per angle
(go.radproj_boxed, go.atom_derivs(boxed=True)): the same sums as the dense
evaluation, cheap enough for the benchmark configurations.
"""
import numpy as np

from . import gauss_oracle as go


def _fields(kind, R, data, bg):
    if kind == "l2":
        return R - data, np.ones_like(R)
    return go.kl_fields(data, R, bg)


def _loss(kind, R, data, bg):
    return go.l2_value(R, data) if kind == "l2" else go.kl_value(data, R, bg)


def _step_params(I, x, r, d, dim, iso):
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


def newton(I, x, r, geom, data, max_iter, kind="l2", bg=0.0, tol=1e-4, min_iter=1):
    I = np.array(I, dtype=np.float64)
    x = np.array(x, dtype=np.float64)
    r = np.array(r, dtype=np.float64).reshape(I.size, -1)
    dim = geom.dim
    iso = r.shape[1] == 1
    n = I.size
    E = np.zeros(max_iter[0] * max_iter[1] * n + 1)
    F = np.zeros_like(E)
    h = [1.0] * n
    eps = 1e-4
    R = go.radproj_boxed(I, x, r, geom)
    F[0] = E[0] = _loss(kind, R, data, bg)
    np.random.seed(1)
    jj = 1
    for it in range(max_iter[0]):
        BREAK = [True, True]
        for j in np.random.permutation(np.arange(n)):
            for _ in range(max_iter[1]):
                BREAK[1] = True
                al, be = _fields(kind, R, data, bg)
                _, df, ddf = go.atom_derivs("field", I[j], x[j], r[j], geom, al, 2, beta=be, boxed=True)
                ddf = ddf + np.eye(df.size) / h[j]
                dx = np.linalg.solve(ddf, -df)
                I1, x1, r1 = _step_params(I[j], x[j], r[j], dx, dim, iso)
                R_old = go.radproj_boxed(I[j:j + 1], x[j:j + 1], r[j:j + 1], geom)
                R_new = go.radproj_boxed(np.array([I1]), x1.reshape(1, -1), r1.reshape(1, -1), geom)
                Rt = R + R_new - R_old
                F[jj] = E[jj] = _loss(kind, Rt, data, bg)
                if E[jj] > E[jj - 1]:
                    E[jj] = E[jj - 1]
                    if h[j] > 2 * eps:
                        BREAK[0] = BREAK[1] = False
                    h[j] /= 10
                else:
                    R = Rt
                    I[j], x[j], r[j] = I1, x1, r1
                    if np.linalg.norm(dx) > tol:
                        BREAK[0] = BREAK[1] = False
                    h[j] *= 2
                h[j] = min(max(h[j], eps), 1 / eps)
                jj += 1
                if BREAK[1]:
                    break
        if BREAK[0] and it > min_iter:
            break
    return (I, x, r), E[:jj], F[:jj]


def _reference_block_grad(df, t, b, D, pr):
    """Block gradient as GD_lib.linesearch_block forms it (GD_lib.py:138-151):
    the slice is chosen by loop position t (df[0], df[1:1+D], df[1+D:]), the
    null regulariser's gradient of block b (shape (1,), (1,D) or (1,pr),
    regularisation.py null.grad) is added with numpy broadcasting, and the
    step is taken along grad[0]."""
    g = df[0] if t == 0 else (df[1:1 + D] if t == 1 else df[1 + D:])
    shape = {"I": (1,), "x": (1, D), "r": (1, pr)}[b]
    g = g + np.zeros(shape)
    return g, g[0]


def gd_block(I, x, r, geom, data, max_iter, kind="l2", bg=0.0, dim_str="xrI", tol=1e-4,
             min_iter=1, slicing="block"):
    """slicing="block": each block steps along its own gradient (the corrected
    rule); slicing="reference": the reference's position-sliced gradient
    (_reference_block_grad), for pinning against the reference's own loop."""
    I = np.array(I, dtype=np.float64)
    x = np.array(x, dtype=np.float64)
    r = np.array(r, dtype=np.float64).reshape(I.size, -1)
    D = geom.dim
    blocks = [b for b, c in (("x", "x"), ("r", "r"), ("I", "i")) if c in dim_str.lower()]
    n = I.size
    E = np.zeros(max_iter[0] * max_iter[1] * n * len(blocks) + 1)
    F = np.zeros_like(E)
    h = [[1e-2] * n for _ in blocks]
    eps = 1e-8
    sl = {"I": slice(0, 1), "x": slice(1, 1 + D), "r": slice(1 + D, None)}
    R = go.radproj_boxed(I, x, r, geom)
    F[0] = E[0] = _loss(kind, R, data, bg)
    np.random.seed(1)
    jj = 1
    for it in range(max_iter[0]):
        BREAK = [True, True]
        for j in np.random.permutation(np.arange(n)):
            for _ in range(max_iter[1]):
                BREAK[1] = True
                for t, b in enumerate(blocks):
                    al, be = _fields(kind, R, data, bg)
                    _, df, _dd = go.atom_derivs("field", I[j], x[j], r[j], geom, al, 1, beta=be,
                                                    boxed=True)
                    if slicing == "reference":
                        grad, step = _reference_block_grad(df, t, b, D, r.shape[1])
                    else:
                        grad = step = df[sl[b]]
                    cur = {"I": np.array([I[j]]), "x": x[j].copy(), "r": r[j].copy()}
                    old = cur[b].copy()
                    h[t][j] = min(h[t][j], 1 / max(np.sqrt((grad * grad).sum()), eps))
                    T = old - h[t][j] * step
                    new = dict(cur)
                    new[b] = T
                    R_old = go.radproj_boxed(I[j:j + 1], x[j:j + 1], r[j:j + 1], geom)
                    R_new = go.radproj_boxed(new["I"], new["x"].reshape(1, -1),
                                       new["r"].reshape(1, -1), geom)
                    Rt = R + R_new - R_old
                    F[jj] = E[jj] = _loss(kind, Rt, data, bg)
                    if E[jj] > E[jj - 1]:
                        E[jj] = E[jj - 1]
                        h[t][j] /= 2
                    else:
                        R = Rt
                        I[j], x[j], r[j] = new["I"][0], new["x"], new["r"]
                        h[t][j] *= 1.1
                        if np.linalg.norm(old - T) > tol * np.linalg.norm(old):
                            BREAK[0] = BREAK[1] = False
                    h[t][j] = max(h[t][j], eps)
                    jj += 1
                if BREAK[1]:
                    break
        if BREAK[0] and it > min_iter:
            break
    return (I, x, r), E[:jj], F[:jj]


def newton_batched(I, x, r, geom, data, iters, kind="l2", bg=0.0, lam0=1.0, lam_min=1e-4,
                   lam_max=1e4, max_backtrack=8):
    """FP64 restatement of the product's all-atoms damped Newton loop."""
    I = np.array(I, dtype=np.float64)
    x = np.array(x, dtype=np.float64)
    r = np.array(r, dtype=np.float64).reshape(I.size, -1)
    dim = geom.dim
    iso = r.shape[1] == 1
    R = go.radproj_boxed(I, x, r, geom)
    loss = _loss(kind, R, data, bg)
    losses = [loss]
    lam = lam0
    for _ in range(iters):
        al, be = _fields(kind, R, data, bg)
        _, g, H = go.all_atom_derivs("field", I, x, r, geom, al, 2, beta=be)
        accepted = False
        for _b in range(max_backtrack):
            In, xn, rn = I.copy(), x.copy(), r.copy()
            for j in range(I.size):
                d = np.linalg.solve(H[j] + lam * np.eye(H.shape[1]), -g[j])
                In[j], xn[j], rn[j] = _step_params(I[j], x[j], r[j], d, dim, iso)
            Rn = go.radproj_boxed(In, xn, rn, geom)
            new = _loss(kind, Rn, data, bg)
            if new <= loss:
                I, x, r, R, loss = In, xn, rn, Rn, new
                lam = min(max(lam / 2, lam_min), lam_max)
                accepted = True
                break
            lam = min(max(lam * 10, lam_min), lam_max)
        losses.append(loss)
        if not accepted:
            break
    return (I, x, r), losses
