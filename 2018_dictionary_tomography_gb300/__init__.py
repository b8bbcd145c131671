"""GB300-native Gaussian-atom Radon engine.

Forward projection of isotropic / anisotropic Gaussian atoms onto 2D and 3D
detectors, and the value, gradient and per-atom Hessian of L2 and KL data
fits, computed by hand-written sm_103a CUDA kernels (csrc/, C ABI in
include/gauss_radon.h) on one GPU.

Drop-in surface of the reference's dictionary/atom API:
  * kernel modules ``NewtonBases2D`` / ``NewtonBases`` with
    ``RadProj, derivs_RadProj, L2derivs_RadProj, VolProj``
    (the plug-in point of GaussDictCode/atomFuncs.py:106-113);
  * ``spaces``: AtomSpace, AtomElement, ProjSpace, ProjElement, VolSpace;
  * ``atomFuncs``: GaussTomo (operator over atoms).
Device-level API: ``engine``.
"""
__version__ = "1.0.0"
