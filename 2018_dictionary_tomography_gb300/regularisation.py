"""Regulariser hook of the fitting loops (GaussDictCode/regularisation.py).

Only ``null`` (:22-37) is provided: the benchmark configurations fit without
a regulariser.  Any object with ``__call__(atoms)``, ``grad(atoms, axis)`` and
``hess(atoms)`` plugs into the loops the same way as in the reference.
"""
import numpy as np


class Regulariser:
    def __init__(self, dim):
        self.dim = dim

    def __call__(self, x):
        return NotImplemented

    def grad(self, x, axis=0):
        return NotImplemented


class null(Regulariser):
    """Value 0, zero gradient and Hessian."""

    def __call__(self, atoms):
        return 0

    def grad(self, atoms, axis=0):
        if axis == 0 or axis == "I":
            return 0 * np.asarray(atoms.I, dtype=np.float64)
        if axis == 1 or axis == "x":
            return 0 * np.asarray(atoms.x, dtype=np.float64)
        if axis == 2 or axis == "r":
            return 0 * np.asarray(atoms.r, dtype=np.float64)
        raise ValueError(axis)

    def hess(self, atoms):
        return 0
