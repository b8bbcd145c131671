"""Drop-in replacement of GaussDictCode/bin/NewtonBases.py (3D and 2.5D).

Same callables and argument meaning as the reference module
(RadProj :714, L2derivs_RadProj :759, derivs_RadProj :954, VolProj :691).
The 2.5D single-axis tilt (two-component orientations with two detector
axes, :685-688) and full 3D frames both run in the sm_103a kernels of
libgauss_radon.so.
"""
from . import _dropin

DIM = 3


def RadProj(atom, Rad, R):
    """Sinogram of all atoms written into R (A, D0, D1) in place."""
    _dropin.radproj(atom, Rad, R, DIM)


def L2derivs_RadProj(atom, Rad, C, order=2):
    """(f, Df, DDf) of 1/2 |R(atom[0]) - C|^2 over the whole sinogram."""
    return _dropin.l2derivs(atom, Rad, C, order, DIM)


def derivs_RadProj(atom, Rad, C, order=2):
    """(f, Df, DDf) of <R(atom[0]), C>: the adjoint (VJP) of the projection."""
    return _dropin.derivs(atom, Rad, C, order, DIM)


def VolProj(atom, y, u):
    """Render the atoms on the voxel grid with coordinate vectors y into u."""
    _dropin.volproj(atom, y, u, DIM)
