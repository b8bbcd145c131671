"""Golden vectors of the reference's regularisers (GaussDictCode/regularisation.py).

Loads that file by path with a stub of its one import
(GaussDictCode.bin.manager.context, whose asarray is numpy's), evaluates
value, gradient (every axis) and, where the reference defines a usable one
(Radius, Iso), the Hessian of seeded atoms one atom at a time, and writes
tests/golden/regularisers.npz.
Needs the reference checkout (run from the repository root):

    python tests/golden/make_reg_golden.py /root/reference
"""
import importlib.util
import os
import sys
import types

import numpy as np


def load_reference(root):
    stub_pkg = types.ModuleType("GaussDictCode")
    stub_bin = types.ModuleType("GaussDictCode.bin")
    stub_mgr = types.ModuleType("GaussDictCode.bin.manager")

    class _Ctx:
        def asarray(self, a):
            return np.asarray(a)
    stub_mgr.context = lambda: _Ctx()
    sys.modules.update({"GaussDictCode": stub_pkg, "GaussDictCode.bin": stub_bin,
                        "GaussDictCode.bin.manager": stub_mgr})
    if not hasattr(np, "infty"):
        np.infty = np.inf       # removed from numpy 2; the reference imports it
    path = os.path.join(root, "GaussDictCode", "regularisation.py")
    spec = importlib.util.spec_from_file_location("ref_regularisation", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class Atoms:
    def __init__(self, I, x, r, iso):
        self.I, self.x, self.r = I, x, r
        self.space = types.SimpleNamespace(isotropic=iso)


def atoms(dim, iso, seed, n=5):
    rng = np.random.default_rng(seed)
    # values on a float32 grid, so the FP32 engine sees the same parameters
    f32 = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)
    I = f32(rng.uniform(0.5, 2.0, n))
    x = f32(rng.uniform(-1, 1, (n, dim)))
    if iso:
        r = f32(rng.uniform(1.5, 3.0, (n, 1)))
    else:
        pr = 3 if dim == 2 else 6
        r = np.concatenate([rng.uniform(1.5, 3.0, (n, dim)), rng.normal(0, 0.7, (n, pr - dim))], 1)
        r = f32(r)
    return Atoms(I, x, r, iso)


def main(root):
    ref = load_reference(root)
    out = {}
    cases = {
        "joubert": lambda d: ref.Joubert(d, 0.7, 0.3, (0.8, 1.3)),
        "mass": lambda d: ref.Mass(d, 0.9, 2, 1.5),
        "volume": lambda d: ref.Volume(d, 1.2, 2, 0.5),
        "radius": lambda d: ref.Radius(d, 0.5, 0.8, 2),
        "iso": lambda d: ref.Iso(d, 0.6),
    }
    sets = []
    for dim in (2, 3):
        for iso in (False, True):
            a = atoms(dim, iso, seed=10 * dim + iso)
            sets.append((dim, iso, "d%d_%s" % (dim, "iso" if iso else "aniso"), a))
            if not iso:
                # the reference's anisotropic Joubert value is +inf as soon as
                # any r entry (off-diagonal ones included) is <= 0: a set with
                # positive off-diagonals pins its finite values
                b = Atoms(a.I, a.x, np.abs(a.r), iso)
                sets.append((dim, iso, "d%d_anisopos" % dim, b))
    for dim, iso, key, a in sets:
        if True:
            out[key + "_I"], out[key + "_x"], out[key + "_r"] = a.I, a.x, a.r
            n = len(a.I)
            for name, make in cases.items():
                reg = make(dim)
                # one atom at a time, as the Newton loop calls them
                # (NewtonGaussian.py:59-66; Mass.grad broadcasts only then)
                vals, grads, hess = [], {0: [], 1: [], 2: []}, []
                for j in range(n):
                    aj = Atoms(a.I[j:j + 1], a.x[j:j + 1], a.r[j:j + 1], iso)
                    with np.errstate(all="ignore"):
                        vals.append(float(reg(aj)))
                        for ax in (0, 1, 2):
                            grads[ax].append(np.asarray(reg.grad(aj, axis=ax),
                                                        dtype=np.float64).reshape(-1))
                        if name in ("radius", "iso"):
                            h = np.asarray(reg.hess(aj), dtype=np.float64)
                            hess.append(h.reshape(h.shape[-2:]))
                out["%s_%s_value" % (key, name)] = np.array(vals)
                for ax in (0, 1, 2):
                    out["%s_%s_grad%d" % (key, name, ax)] = np.stack(grads[ax])
                if hess:
                    out["%s_%s_hess" % (key, name)] = np.stack(hess)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "regularisers.npz")
    np.savez(dst, **out)
    print("wrote", dst, len(out), "arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
