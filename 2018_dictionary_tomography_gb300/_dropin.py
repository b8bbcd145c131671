"""Shared implementation of the drop-in kernel modules.

The reference's kernel modules (GaussDictCode/bin/NewtonBases2D.py,
GaussDictCode/bin/NewtonBases.py) expose four callables that GaussTomo
dispatches to (GaussDictCode/atomFuncs.py:106-113):

  RadProj(atom, Rad, R)                  writes the sinogram into R in place
  L2derivs_RadProj(atom, Rad, C, order)  (f, Df, DDf) of 1/2|R(atom[0]) - C|^2
  derivs_RadProj(atom, Rad, C, order)    (f, Df, DDf) of <R(atom[0]), C>
  VolProj(atom, y, u)                    renders atoms on a voxel grid

Arguments are duck-typed as in the reference: ``atom`` has I, x, r (numpy or
torch); ``Rad.range`` has orientations, ortho, detector; C is an array or has
``asarray()``.  Host arrays are copied to the GPU; CUDA tensors are used in
place.  The derivative callables take the first atom, as the reference's do
(they read atom.I[0], atom.x[0], atom.r[0]), and return float64 host arrays
(the reference returns float32).  Isotropic atoms give P = 2 + d parameters
with the exact chain rule of r = (s, .., s, 0, ..).
"""
import weakref

import numpy as np
import torch

from . import engine
from .geometry import DeviceGeometry

_geoms = weakref.WeakKeyDictionary()


def _space_geometry(space):
    try:
        g = _geoms.get(space)
    except TypeError:
        g = None
    if g is None:
        g = DeviceGeometry(space.orientations, space.ortho, space.detector)
        try:
            _geoms[space] = g
        except TypeError:
            pass
    return g


def _atoms(atom, first_only=False):
    I, x, r = atom.I, atom.x, atom.r
    if first_only:
        I, x, r = I[:1], x[:1], r[:1]
    return engine.DeviceAtoms(_tensor(I), _tensor(x), _tensor(r))


def _tensor(a):
    if isinstance(a, torch.Tensor):
        return a
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np.float32))


def _data(C):
    if hasattr(C, "asarray"):
        C = C.asarray()
    return C


def radproj(atom, Rad, R, dim, psf=False):
    geom = _space_geometry(Rad.range)
    if dim is not None and geom.dim != dim:
        raise ValueError("this kernel module handles %dD geometry" % dim)
    atoms = _atoms(atom)
    if isinstance(R, torch.Tensor) and R.is_cuda:
        if R.dtype == torch.float32 and R.is_contiguous():
            engine.radproj(atoms, geom, out=R, psf=psf)
        else:
            R.copy_(engine.radproj(atoms, geom, psf=psf))
        return
    out = engine.radproj(atoms, geom, psf=psf)
    host = out.cpu().numpy()
    if isinstance(R, torch.Tensor):
        R.copy_(torch.from_numpy(host))
    else:
        R[...] = host.reshape(np.shape(R))


def _derivs(atom, Rad, C, order, mode, dim, psf=False):
    geom = _space_geometry(Rad.range)
    if dim is not None and geom.dim != dim:
        raise ValueError("this kernel module handles %dD geometry" % dim)
    atoms = _atoms(atom, first_only=True)
    C = _tensor(_data(C))
    o = 2 if order > 1 else 1
    f, g, H = engine.atom_derivs(atoms, geom, mode, C.reshape(geom.shape), order=o, psf=psf)
    f = float(f[0].item())
    Df = g[0].cpu().numpy()
    DDf = H[0].cpu().numpy() if H is not None else np.zeros((Df.size, Df.size))
    return f, Df, DDf


def l2derivs(atom, Rad, C, order, dim, psf=False):
    return _derivs(atom, Rad, C, order, "l2_atom", dim, psf)


def derivs(atom, Rad, C, order, dim, psf=False):
    return _derivs(atom, Rad, C, order, "inner", dim, psf)


def volproj(atom, y, u, dim, psf=False):
    from . import volume
    volume.volproj_into(_atoms(atom), y, u, dim, psf=psf)
