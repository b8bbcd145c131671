"""GaussTomo: the Gaussian-atom Radon operator over an AtomSpace.

Mirrors GaussDictCode/atomFuncs.py: ``GaussTomo`` (:77) with ``_getOps``
(:106, the kernel-module plug-in point), ``__call__`` (:115), ``discretise``
(:121), ``derivs`` (:130), ``gradient`` (:144) and ``L2_derivs`` (:146), and
``SingleParticleGaussTomo`` (:161).  The reference loops over atoms in Python
and launches one kernel per atom; here ``derivs`` and ``L2_derivs`` evaluate
every atom in one engine call with the same per-atom semantics (each atom
against the same C), and return the same stacked arrays:
f (N, 1), df (N, P), ddf (N, P, P).
"""
import importlib

import numpy as np
import torch

from . import engine, spaces
from .geometry import DeviceGeometry


class GaussTomo:
    """Operator atoms -> sinogram on ``Sino`` (a ProjSpace)."""

    def __init__(self, Atoms, Volume, Sino, device="GPU"):
        self.domain = Atoms
        self.range = Sino
        self.embedding = Volume
        self._device = device.lower()
        if self._device == "cpu":
            # same error as the reference (atomFuncs.py:95-96): there is no CPU path
            raise ValueError("CPU processing not yet supported")
        (self._fwrd, self._derivs_op, self._l2derivs_op,
         self._proj) = self._getOps(Atoms.dim)
        self._geom = None

    _psf = False

    def _getOps(self, dim):
        pkg = __name__.rsplit(".", 1)[0]
        if dim == 2:
            mod = importlib.import_module(pkg + ".NewtonBases2D")
        elif dim == 3:
            mod = importlib.import_module(pkg + ".NewtonBases")
        else:
            raise ValueError
        return mod.RadProj, mod.derivs_RadProj, mod.L2derivs_RadProj, mod.VolProj

    # ---- device geometry (cached) --------------------------------------
    @property
    def geometry(self):
        if self._geom is None:
            S = self.range
            self._geom = DeviceGeometry(S.orientations, S.ortho, S.detector)
        return self._geom

    def device_atoms(self, atoms):
        return engine.DeviceAtoms(_t(atoms.I), _t(atoms.x), _t(atoms.r))

    # ---- reference operator API ------------------------------------------
    def __call__(self, atoms, out=None):
        if out is None:
            out = self.range.element(np.empty(self.range.shape, dtype=np.float32))
        self._fwrd(atoms, self, out.data)
        return out

    def discretise(self, atoms, out=None):
        if out is None:
            out = self.embedding.element(np.empty(self.embedding.shape, dtype=np.float32))
        self._proj(atoms, self.embedding.coord_vectors, out.data)
        return out

    def _stackAtoms(self, atoms):
        return self.domain.element(np.vstack(atoms))

    def _derivs_all(self, atoms, C, order, mode):
        C = C.asarray() if hasattr(C, "asarray") else C
        field = C if isinstance(C, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(C, dtype=np.float32))
        f, g, H = engine.atom_derivs(self.device_atoms(atoms), self.geometry, mode,
                                     field.reshape(self.geometry.shape),
                                     order=2 if order > 1 else 1, psf=self._psf)
        f = f.cpu().numpy().reshape(-1, 1)
        df = g.cpu().numpy()
        if order == 1:
            return f, df
        return f, df, H.cpu().numpy()

    def derivs(self, atoms, C, order=2):
        """Per atom: <R(a), C>, <dR(a), C>, <d2R(a), C> (atomFuncs.py:130)."""
        return self._derivs_all(atoms, C, order, "inner")

    def gradient(self, x):
        """Linear map d -> d<R(x), d>/dx per atom (atomFuncs.py:144)."""
        op = self

        class _Gradient:
            def __call__(self, d):
                return op.derivs(x, d, order=1)[1]
        return _Gradient()

    def L2_derivs(self, atoms, C, order=2):
        """Per atom: value, gradient, Hessian of 1/2|R(a) - C|^2
        (atomFuncs.py:146)."""
        return self._derivs_all(atoms, C, order, "l2_atom")


class SingleParticleGaussTomo(GaussTomo):
    """GaussTomo with the pixel-integrated point-spread kernels
    (atomFuncs.py:161-172)."""

    _psf = True

    def _getOps(self, dim):
        if dim not in (2, 3):
            raise ValueError
        pkg = __name__.rsplit(".", 1)[0]
        mod = importlib.import_module(pkg + ".point_spread_functions")
        return mod.RadProj, mod.derivs_RadProj, mod.L2derivs_RadProj, mod.VolProj


def _t(a):
    if isinstance(a, torch.Tensor):
        return a
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))


def theta_to_vec(theta):
    from .geometry import theta_to_vec as t2v
    return t2v(theta)


def perp(theta):
    from .geometry import perp as p
    return p(theta)
