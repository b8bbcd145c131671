"""The FP64 fitting-loop oracle (test infrastructure) checked on the CPU:
its accept rules keep the energy from rising, its fits improve a jittered
start, and its parameter update applies the reference's clamps
(GD_lib.py:504-522).  The GPU tests compare the product's loops against it."""
import numpy as np
import pytest

from oracle import fit_oracle
from oracle import gauss_oracle as go
from problems import make_atoms, make_geometry


def _problem(kind, seed=3, N=5):
    g = make_geometry("2d", 12, 40)
    I, x, r = make_atoms(2, N, seed, rdiag=(4.0, 7.0), roff=0.5, box=0.5)
    R = go.radproj(I, x, r, g)
    data = R + (0.5 if kind == "kl" else 0.0)
    rng = np.random.default_rng(seed + 100)
    x0 = x + rng.normal(0, 0.02, x.shape)
    I0 = I * rng.uniform(0.9, 1.1, I.shape)
    return g, data, (I0, x0, r.copy())


@pytest.mark.parametrize("kind", ["l2", "kl"])
def test_batched_newton_oracle_never_raises_the_loss(kind):
    g, data, (I0, x0, r0) = _problem(kind)
    bg = 0.5 if kind == "kl" else 0.0
    _, losses = fit_oracle.newton_batched(I0, x0, r0, g, data, 6, kind, bg)
    assert len(losses) >= 2
    assert all(b <= a for a, b in zip(losses, losses[1:]))
    assert losses[-1] < 0.9 * losses[0]


def test_per_atom_newton_oracle_energy_is_monotone():
    g, data, (I0, x0, r0) = _problem("l2")
    (I, x, r), E, F = fit_oracle.newton(I0, x0, r0, g, data, [3, 2], "l2")
    assert E.size >= 2 and F.size == E.size
    assert np.all(np.diff(E) <= 0)
    # the energy of the returned atoms is the last accepted one
    assert abs(go.l2_value(go.radproj(I, x, r, g), data) - E[-1]) <= 1e-9 * E[0]
    assert E[-1] < E[0]


def test_block_gd_oracle_energy_is_monotone():
    g, data, (I0, x0, r0) = _problem("l2", seed=7)
    _, E, _F = fit_oracle.gd_block(I0, x0, r0, g, data, [3, 1])
    assert np.all(np.diff(E) <= 0)
    assert E[-1] <= E[0]


def test_step_clamps_follow_the_reference():
    # I stays >= 0; a negative diagonal entry of r flips the sign of its row
    I, x, r = 0.3, np.zeros(2), np.array([2.0, 3.0, 0.5])
    d = np.array([-1.0, 0.1, -0.2, -5.0, -4.0, 0.25])
    I1, x1, r1 = fit_oracle._step_params(I, x, r, d, 2, False)
    assert I1 == 0.0
    assert np.allclose(x1, [0.1, -0.2])
    # r + d = [-3, -1, 0.75]: row 0 flips (r00, r01), row 1 flips r11
    assert np.allclose(r1, [3.0, 1.0, -0.75])
    r3 = np.array([1.0, 1.0, 1.0, 0.1, 0.2, 0.3])
    d3 = np.concatenate([[0.0], np.zeros(3), [-2.0, 0.0, -3.0, 0.0, 0.0, 0.0]])
    _, _, r31 = fit_oracle._step_params(1.0, np.zeros(3), r3, d3, 3, False)
    # rows 0 (r00 r01 r02) and 2 (r22) flip
    assert np.allclose(r31, [1.0, 1.0, 2.0, -0.1, 0.2, -0.3])
    _, _, ri = fit_oracle._step_params(1.0, np.zeros(2), np.array([2.0]), np.array([0, 0, 0, -3.0]),
                                       2, True)
    assert np.allclose(ri, [1.0])
