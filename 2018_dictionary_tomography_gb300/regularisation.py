"""Regularisers of the fitting loops (GaussDictCode/regularisation.py).

Same classes and call protocol as the reference -- ``reg(atoms)`` (total
value), ``reg.grad(atoms, axis)`` and ``reg.hess(atoms)`` -- for ``null``
(:22-37), ``Joubert`` (:41-107), ``Mass`` (:110-208), ``Volume`` (:211-297),
``Radius`` (:300-366) and ``Iso`` (:369-442).  Every non-null regulariser is
evaluated on the GPU by ``gr_regulariser`` (one thread per atom, FP64), and
``device_terms`` adds the terms of every atom to the outputs of the
derivative kernels in one launch, for the batched Newton step.

Differences from the reference (the oracle, oracle/reg_oracle.py, follows
these and is checked against the reference's own values and gradients):
  * ``grad(atoms)`` defaults to ``axis=None`` (the concatenation
    ``[dI, dx, dr]``) for every class; the reference's Joubert defaults to
    ``axis=0``, which its Newton loop then broadcasts over the whole block;
  * the anisotropic Joubert value needs a positive diagonal of r only (the
    reference returns +inf when any entry of r is <= 0);
  * Volume's gradient includes the factor k of d/dr |R - v0|^k;
  * Hessians are exact for every class and returned per atom (N, P, P).
"""
import numpy as np
import torch

from . import engine


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
        if axis is None:
            return np.concatenate([0 * np.asarray(a, dtype=np.float64).reshape(-1)
                                   for a in (atoms.I, atoms.x, atoms.r)])
        raise ValueError(axis)

    def hess(self, atoms):
        return 0

    def device_terms(self, atoms, f, g, H):
        return f, g, H


def _device_atoms(atoms):
    if isinstance(atoms, engine.DeviceAtoms):
        return atoms
    t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float32))
    return engine.DeviceAtoms(t(atoms.I), t(atoms.x), t(atoms.r))


class _DeviceRegulariser(Regulariser):
    """A regulariser evaluated by the ``gr_regulariser`` kernel."""

    kind = None

    def __init__(self, dim, params, scale=1.0):
        super().__init__(dim)
        self.params = tuple(float(p) for p in params)
        self.scale = float(scale)

    def _p(self):
        """Kernel parameters with the scale folded into the weight."""
        raise NotImplementedError

    def terms(self, atoms, order=2):
        """Per-atom value (N,), gradient (N, P), Hessian (N, P, P) as FP64
        device tensors."""
        return engine.regulariser(self.kind, self._p(), _device_atoms(atoms), order=order)

    def device_terms(self, atoms, f, g, H):
        """Add every atom's value, gradient and Hessian to f, g, H."""
        engine.regulariser(self.kind, self._p(), atoms, f, g, H, accumulate=True,
                           order=2 if H is not None else 1)
        return f, g, H

    def __call__(self, atoms):
        f, _, _ = self.terms(atoms, order=1)
        return float(f.sum().item())

    def grad(self, atoms, axis=None):
        _, g, _ = self.terms(atoms, order=1)
        g = g.cpu().numpy()
        d = self.dim
        if axis == 0 or axis == "I":
            return g[:, 0]
        if axis == 1 or axis == "x":
            return g[:, 1:1 + d]
        if axis == 2 or axis == "r":
            return g[:, 1 + d:]
        if axis is None:
            return np.concatenate([g[:, 0].reshape(-1), g[:, 1:1 + d].reshape(-1),
                                   g[:, 1 + d:].reshape(-1)])
        raise ValueError(axis)

    def hess(self, atoms):
        _, _, H = self.terms(atoms, order=2)
        return H.cpu().numpy()

    def __mul__(self, scal):
        if np.isscalar(scal):
            out = object.__new__(type(self))
            out.__dict__.update(self.__dict__)
            out.scale = self.scale * float(scal)
            return out
        return NotImplemented

    __rmul__ = __mul__


class Joubert(_DeviceRegulariser):
    """-a log I + b/2 |x|^2 + c R - d log R - e, R = prod(diag r) (or s^dim):
    the reference's Joubert(dim, intensity, location, radius)."""

    kind = "joubert"

    def __init__(self, dim, intensity, location, radius):
        r0, r1 = float(radius[0]), float(radius[1])
        super().__init__(dim, (intensity, location, r1, r1 * r0, r0 * r1 * (1 - np.log(r0))))

    def _p(self):
        return tuple(self.scale * p for p in self.params)


class Mass(_DeviceRegulariser):
    """s (I V - m)^k, V = I / det(r) (or I s^dim)."""

    kind = "mass"

    def __init__(self, dim, m, k=2, s=1):
        super().__init__(dim, (m, k, s))

    def _p(self):
        m, k, s = self.params
        return (m, k, s * self.scale)


class Volume(_DeviceRegulariser):
    """s |det(r) - r0^dim|^k (isotropic: det = s^-dim)."""

    kind = "volume"

    def __init__(self, dim, r0, k=2, s=1):
        super().__init__(dim, (abs(r0) ** dim, k, s))

    def _p(self):
        v0, k, s = self.params
        return (v0, k, s * self.scale)


class Radius(_DeviceRegulariser):
    """s sum (r_ii - r0)^-k over the diagonal of r (isotropic: dim (s - r0)^-k)."""

    kind = "radius"

    def __init__(self, dim, r0, s, k):
        super().__init__(dim, (r0, s, k))

    def _p(self):
        r0, s, k = self.params
        return (r0, s * self.scale, k)


class Iso(_DeviceRegulariser):
    """s/2 |off-diagonal r|^2: pulls anisotropic atoms towards isotropy."""

    kind = "iso"

    def __init__(self, dim, s):
        super().__init__(dim, (s,))

    def _p(self):
        return (self.params[0] * self.scale,)
