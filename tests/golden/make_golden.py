"""Regenerate the known-answer vectors for the per-pixel atom derivatives.

The reference pins its derivative formulas only through the sympy self-tests
in GaussDictCode/bin/NewtonBases2D.py:518-583 and
GaussDictCode/bin/NewtonBases.py:1155-1229.  Those blocks differentiate
1/2 (I * basis(|M r (y - x)|^2) / |r T| - C)^2 symbolically with respect to
(I, x, r) but use the stale basis exp(-n/2); the kernels use exp(-30 n)
(NewtonBases.py:50-71).  This script rebuilds the same symbolic expression
with the kernels' basis and evaluates value, gradient and Hessian at seeded
points, including the 2.5D point the 3D self-test uses (T = (1, 1, 0),
y = (1, -1, 3), NewtonBases.py:1185-1187).

Run:  python tests/golden/make_golden.py   (writes tests/golden/pointwise.npz)
"""
import os

import numpy as np
import sympy as sp


def symbolic(dim):
    nr = 3 if dim == 2 else 6
    I = sp.Symbol("I", real=True)
    x = sp.symbols("x:%d" % dim, real=True)
    y = sp.symbols("y:%d" % dim, real=True)
    r = sp.symbols("r:%d" % nr, real=True)
    T = sp.symbols("T:%d" % dim, real=True)
    C = sp.Symbol("C", real=True)
    Y = [y[i] - x[i] for i in range(dim)]
    if dim == 2:
        rY = (r[0] * Y[0] + r[2] * Y[1], r[1] * Y[1])
        rT = (r[0] * T[0] + r[2] * T[1], r[1] * T[1])
    else:
        rY = (r[0] * Y[0] + r[3] * Y[1] + r[5] * Y[2], r[1] * Y[1] + r[4] * Y[2], r[2] * Y[2])
        rT = (r[0] * T[0] + r[3] * T[1] + r[5] * T[2], r[1] * T[1] + r[4] * T[2], r[2] * T[2])
    nT = sp.sqrt(sum(t ** 2 for t in rT))
    ip = sum(a * b for a, b in zip(rY, rT)) / nT
    MY = [rY[i] - ip * rT[i] / nT for i in range(dim)]
    m = sum(v ** 2 for v in MY)
    Rf = I * sp.exp(-30 * m) / nT
    F = (Rf - C) ** 2 / 2
    var = (I,) + tuple(x) + tuple(r)
    dF = [sp.diff(F, v) for v in var]
    ddF = [[sp.diff(d, v) for v in var] for d in dF]
    args = (C, I) + tuple(x) + tuple(y) + tuple(r) + tuple(T)
    fn = sp.lambdify(args, [Rf, m, F, dF, ddF], "mpmath")
    return fn


def main():
    import mpmath
    mpmath.mp.dps = 30
    rng = np.random.RandomState(0)
    cases = []
    for dim in (2, 3):
        fn = symbolic(dim)
        nr = 3 if dim == 2 else 6
        k = 0
        while k < 6:
            I = rng.rand(1) + 0.5
            x = rng.rand(dim) * 0.4 - 0.2
            r = np.concatenate([rng.rand(dim) * 3 + 1.5, rng.randn(nr - dim) * 0.8])
            T = rng.randn(dim)
            T /= np.linalg.norm(T)
            y = x + rng.randn(dim) * 0.12
            C = rng.rand(1)
            lenT = dim
            if dim == 3 and k == 5:
                # the 2.5D point of the reference self-test
                T = np.array([1.0, 1.0, 0.0])
                y = np.array([1.0, -1.0, 3.0])
                x = np.array([0.9, -0.8, 2.95])
                lenT = 2
            vals = fn(C[0], I[0], *x, *y, *r, *T)
            Rf, m = float(vals[0]), float(vals[1])
            if m > 0.9:   # keep known answers strictly inside the support
                continue
            F = float(vals[2])
            dF = np.array([float(v) for v in vals[3]])
            ddF = np.array([[float(v) for v in row] for row in vals[4]])
            cases.append(dict(dim=dim, lenT=lenT, I=I[0], x=x, r=r, T=T, y=y, C=C[0],
                              R=Rf, m=m, F=F, dF=dF, ddF=ddF))
            k += 1
    out = {}
    for i, c in enumerate(cases):
        for key, v in c.items():
            out["c%d_%s" % (i, key)] = np.asarray(v)
    out["n"] = np.asarray(len(cases))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pointwise.npz")
    np.savez(path, **out)
    print("wrote", path, len(cases), "cases")


if __name__ == "__main__":
    main()
