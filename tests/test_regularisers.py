"""Per-atom regularisers: the FP64 oracle against golden values and gradients
of the reference's own regularisation.py (tests/golden/make_reg_golden.py),
and its exact Hessians against central differences of its gradients.
CPU only."""
import os

import numpy as np
import pytest

from oracle import reg_oracle as ro

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "regularisers.npz"))

# the generator's constructors, as oracle parameters per dimension
PARAMS = {
    "joubert": lambda d: ro.joubert_params(0.7, 0.3, (0.8, 1.3)),
    "mass": lambda d: (0.9, 2.0, 1.5),
    "volume": lambda d: (1.2 ** d, 2.0, 0.5),
    "radius": lambda d: (0.5, 0.8, 2.0),
    "iso": lambda d: (0.6,),
}
SETS = ["d2_aniso", "d2_anisopos", "d2_iso", "d3_aniso", "d3_anisopos", "d3_iso"]


def _set(key):
    dim = int(key[1])
    iso = key.endswith("_iso")
    return dim, iso, GOLD[key + "_I"], GOLD[key + "_x"], GOLD[key + "_r"]


@pytest.mark.parametrize("key", SETS)
@pytest.mark.parametrize("kind", list(PARAMS))
def test_oracle_matches_reference_values_and_gradients(key, kind):
    dim, iso, I, x, r = _set(key)
    f, g, H = ro.terms(kind, PARAMS[kind](dim), I, x, r, dim, iso)
    gv = GOLD["%s_%s_value" % (key, kind)]
    if kind == "joubert" and not iso and key.endswith("_aniso"):
        # the reference returns +inf when any r entry (off-diagonal ones
        # included) is <= 0; ours only needs a positive diagonal
        neg_off = np.any(r[:, dim:] <= 0, axis=1)
        assert np.all(np.isinf(gv[neg_off])) and np.all(np.isfinite(f))
        gv, f = gv[~neg_off], f[~neg_off]
    np.testing.assert_allclose(f, gv, rtol=1e-12, atol=0)
    dI, dx, dr = g[:, :1], g[:, 1:1 + dim], g[:, 1 + dim:]
    kfac = 2.0 if kind == "volume" else 1.0   # the reference's Volume gradient lacks the factor k
    np.testing.assert_allclose(dI, GOLD["%s_%s_grad0" % (key, kind)].reshape(dI.shape), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(dx, GOLD["%s_%s_grad1" % (key, kind)].reshape(dx.shape), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(dr, kfac * GOLD["%s_%s_grad2" % (key, kind)].reshape(dr.shape),
                               rtol=1e-12, atol=1e-14)
    hk = "%s_%s_hess" % (key, kind)
    if hk in GOLD.files:
        np.testing.assert_allclose(H, GOLD[hk], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("key", SETS)
@pytest.mark.parametrize("kind", list(PARAMS))
def test_oracle_hessian_is_the_derivative_of_its_gradient(key, kind):
    dim, iso, I, x, r = _set(key)
    p = PARAMS[kind](dim)
    h = 1e-6
    for j in range(len(I)):
        th = np.concatenate([[I[j]], x[j], r[j]])
        _, g0, H0 = ro.atom_terms(kind, p, th[0], th[1:1 + dim], th[1 + dim:], dim, iso)
        P = len(th)
        Hfd = np.zeros((P, P))
        for a in range(P):
            tp, tm = th.copy(), th.copy()
            tp[a] += h
            tm[a] -= h
            gp = ro.atom_terms(kind, p, tp[0], tp[1:1 + dim], tp[1 + dim:], dim, iso)[1]
            gm = ro.atom_terms(kind, p, tm[0], tm[1:1 + dim], tm[1 + dim:], dim, iso)[1]
            Hfd[:, a] = (gp - gm) / (2 * h)
        scale = max(1.0, np.abs(H0).max())
        assert np.abs(Hfd - H0).max() <= 1e-6 * scale
        # and the gradient is the derivative of the value
        if np.isfinite(ro.atom_terms(kind, p, th[0], th[1:1 + dim], th[1 + dim:], dim, iso)[0]):
            for a in range(P):
                tp, tm = th.copy(), th.copy()
                tp[a] += h
                tm[a] -= h
                fp = ro.atom_terms(kind, p, tp[0], tp[1:1 + dim], tp[1 + dim:], dim, iso)[0]
                fm = ro.atom_terms(kind, p, tm[0], tm[1:1 + dim], tm[1 + dim:], dim, iso)[0]
                if kind == "mass":
                    continue    # the value takes |V|, the gradient (V - m): equal for V > 0 only
                assert abs((fp - fm) / (2 * h) - g0[a]) <= 1e-6 * max(1.0, abs(g0[a]))
