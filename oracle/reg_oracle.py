"""FP64 oracle of the per-atom regularisers (test infrastructure only).

Restates the regularisers of GaussDictCode/regularisation.py -- Joubert
(:41-107), Mass (:110-208), Volume (:211-297), Radius (:300-366), Iso
(:369-442) -- per atom in numpy: value, gradient and Hessian in the
parameter order [I, x, r].  Corrected semantics, checked against the
reference's own values and gradients in tests/golden/regularisers.npz:
  * an anisotropic Joubert value is finite whenever I and the diagonal of r
    are positive (the reference returns +inf as soon as any r entry,
    off-diagonal ones included, is <= 0);
  * Hessians are exact second derivatives (Joubert has none in the
    reference, Volume's cannot run, Mass's misses mixed r-r terms); they are
    checked against central differences of the gradients.
Only the tests use this module.
"""
import numpy as np


def n_params(dim, iso):
    return 1 + dim + (1 if iso else (3 if dim == 2 else 6))


def joubert_params(intensity, location, radius):
    """(a, b, c, d, e) of the reference's Joubert(dim, intensity, location, radius)."""
    return (intensity, location, radius[1], radius[1] * radius[0],
            radius[0] * radius[1] * (1 - np.log(radius[0])))


def _diag_product(r, dim, iso):
    return r[0] ** dim if iso else np.prod(r[:dim])


def atom_terms(kind, p, I, x, r, dim, iso):
    """value, gradient (P,), Hessian (P, P) of one atom."""
    P = n_params(dim, iso)
    g = np.zeros(P)
    H = np.zeros((P, P))
    r0 = 1 + dim
    r = np.asarray(r, dtype=np.float64).reshape(-1)
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    nd = 1 if iso else dim
    if kind == "null":
        return 0.0, g, H
    if kind == "joubert":
        a, b, c, d, e = p
        R = _diag_product(r, dim, iso)
        ok = I > 0 and np.all(r[:nd] > 0)
        val = (-a * np.log(I) + b / 2 * x @ x + c * R - d * np.log(R) - e) if ok else np.inf
        g[0], H[0, 0] = -a / I, a / I ** 2
        g[1:1 + dim] = b * x
        H[1:1 + dim, 1:1 + dim] = b * np.eye(dim)
        if iso:
            s = r[0]
            g[r0] = dim * c * s ** (dim - 1) - dim * d / s
            H[r0, r0] = dim * (dim - 1) * c * s ** (dim - 2) + dim * d / s ** 2
        else:
            for i in range(dim):
                g[r0 + i] = (c * R - d) / r[i]
                for k in range(dim):
                    H[r0 + i, r0 + k] = d / r[i] ** 2 if i == k else c * R / (r[i] * r[k])
        return val, g, H
    if kind == "mass":
        m, k, w = p
        if iso:
            Rv = r[0] ** dim
        else:
            Rv = 1.0 / np.prod(r[:dim])
        V = I * Rv
        dV = np.zeros(P)
        d2V = np.zeros((P, P))
        dV[0] = Rv
        if iso:
            s = r[0]
            dV[r0] = dim * I * s ** (dim - 1)
            d2V[0, r0] = d2V[r0, 0] = dim * s ** (dim - 1)
            d2V[r0, r0] = dim * (dim - 1) * I * s ** (dim - 2)
        else:
            for i in range(dim):
                dV[r0 + i] = -V / r[i]
                d2V[0, r0 + i] = d2V[r0 + i, 0] = -Rv / r[i]
                for t in range(dim):
                    d2V[r0 + i, r0 + t] = (2.0 if i == t else 1.0) * V / (r[i] * r[t])
        u = V - m
        with np.errstate(all="ignore"):
            val = np.inf if I < 0 else w * (abs(V) - m) ** k
            s1 = w * k * u ** (k - 1)
            s2 = w * k * (k - 1) * u ** (k - 2)
        return val, s1 * dV, s2 * np.outer(dV, dV) + s1 * d2V
    if kind == "volume":
        v0, k, w = p
        dR = np.zeros(nd)
        d2R = np.zeros((nd, nd))
        if iso:
            s = r[0]
            ok = s > 0
            R = s ** -dim
            dR[0] = -dim * s ** (-dim - 1)
            d2R[0, 0] = dim * (dim + 1) * s ** (-dim - 2)
        else:
            ok = np.all(r[:dim] > 0)
            R = np.prod(r[:dim])
            for i in range(dim):
                dR[i] = R / r[i]
                for t in range(dim):
                    d2R[i, t] = 0.0 if i == t else R / (r[i] * r[t])
        u = R - v0
        with np.errstate(all="ignore"):
            val = w * abs(u) ** k if ok else np.inf
            s1 = w * k * np.sign(u) * abs(u) ** (k - 1)
            s2 = w * k * (k - 1) * abs(u) ** (k - 2)
        g[r0:r0 + nd] = s1 * dR
        H[r0:r0 + nd, r0:r0 + nd] = s2 * np.outer(dR, dR) + s1 * d2R
        return val, g, H
    if kind == "radius":
        rr0, w, k = p
        mult = dim if iso else 1
        t = r[:nd] - rr0
        with np.errstate(all="ignore"):
            val = w * mult * np.sum(t ** -k) if np.all(t > 0) else np.inf
            g[r0:r0 + nd] = w * mult * (-k) * t ** (-k - 1)
            H[r0:r0 + nd, r0:r0 + nd] = np.diag(w * mult * k * (k + 1) * t ** (-k - 2))
        return val, g, H
    if kind == "iso":
        (w,) = p[:1]
        if iso:
            return 0.0, g, H
        off = r[dim:]
        g[r0 + dim:] = w * off
        H[r0 + dim:, r0 + dim:] = w * np.eye(len(off))
        return 0.5 * w * off @ off, g, H
    raise ValueError(kind)


def terms(kind, p, I, x, r, dim, iso):
    """Per-atom values (N,), gradients (N, P), Hessians (N, P, P)."""
    I = np.asarray(I, dtype=np.float64).reshape(-1)
    n = len(I)
    x = np.asarray(x, dtype=np.float64).reshape(n, -1)
    r = np.asarray(r, dtype=np.float64).reshape(n, -1)
    out = [atom_terms(kind, p, I[j], x[j], r[j], dim, iso) for j in range(n)]
    return (np.array([o[0] for o in out]), np.stack([o[1] for o in out]),
            np.stack([o[2] for o in out]))
