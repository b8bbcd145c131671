"""Drop-in replacement of GaussDictCode/bin/point_spread_functions.py.

The single-particle kernel module that SingleParticleGaussTomo selects
(GaussDictCode/atomFuncs.py:168-172): pixel-integrated projections of atoms,
their derivatives, and voxel-integrated renderings, for 2D, 2.5D and 3D
geometry.  Same callables and argument meaning as the reference (RadProj
:371, L2derivs_RadProj :1077, derivs_RadProj :1314, VolProj :168); the work
runs in the sm_103a kernels of libgauss_radon.so (gr_psf_* entry points).
"""
from . import _dropin


def RadProj(atom, Rad, R):
    """Pixel-integrated sinogram of all atoms written into R in place."""
    _dropin.radproj(atom, Rad, R, None, psf=True)


def L2derivs_RadProj(atom, Rad, C, order=2):
    """(f, Df, DDf) of 1/2 |R_pix(atom[0]) - C|^2 over the whole sinogram."""
    return _dropin.l2derivs(atom, Rad, C, order, None, psf=True)


def derivs_RadProj(atom, Rad, C, order=2):
    """(f, Df, DDf) of <R_pix(atom[0]), C>."""
    return _dropin.derivs(atom, Rad, C, order, None, psf=True)


def VolProj(atom, y, u):
    """Voxel-integrated rendering of the atoms into u."""
    _dropin.volproj(atom, y, u, len(y), psf=True)
