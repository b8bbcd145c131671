"""Drop-in replacement of GaussDictCode/bin/NewtonBases2D.py (2D atoms).

Same callables and argument meaning as the reference module
(RadProj :274, L2derivs_RadProj :299, derivs_RadProj :415, VolProj :252);
the work runs in the sm_103a kernels of libgauss_radon.so.
"""
from . import _dropin

DIM = 2


def RadProj(atom, Rad, R):
    """Sinogram of all atoms written into R (A, D) in place."""
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
