"""Rendering atoms on voxel grids (GaussTomo.discretise / VolProj)."""
import ctypes

import numpy as np
import torch

from . import _lib, engine


def volproj(atoms, coords, device=None, psf=False):
    """u (V0, V1[, V2]) float32 on the device for an engine.DeviceAtoms and
    coordinate vectors ``coords`` (one 1-D array per axis).  psf=True gives
    voxel integrals (half-width = half the spacing of axis 1, as the
    reference's point-spread VolProj assumes)."""
    dev = atoms.I.device if atoms.n else torch.device(device or "cuda")
    dim = len(coords)
    if atoms.n and atoms.dim != dim:
        raise ValueError("atoms are %dD, grid is %dD" % (atoms.dim, dim))
    ys = [torch.as_tensor(np.asarray(c, dtype=np.float32).reshape(-1) if not isinstance(c, torch.Tensor)
                          else c.float().reshape(-1)).to(dev).contiguous() for c in coords]
    shape = tuple(int(y.numel()) for y in ys)
    u = torch.empty(shape, dtype=torch.float32, device=dev)
    n = (ctypes.c_int * 3)(*(list(shape) + [1] * (3 - dim)))
    ptrs = (ctypes.c_void_p * 3)(*([y.data_ptr() for y in ys] + [None] * (3 - dim)))
    if psf:
        c1 = np.asarray(coords[1] if not isinstance(coords[1], torch.Tensor)
                        else coords[1].cpu().numpy(), dtype=np.float64).reshape(-1)
        s = abs(float(c1[1] - c1[0])) / 2
        st = _lib.load().gr_psf_volproj(ctypes.byref(atoms.struct), dim,
                                        ctypes.cast(n, ctypes.c_void_p),
                                        ctypes.cast(ptrs, ctypes.c_void_p), s, u.data_ptr(),
                                        engine._stream_handle(dev))
    else:
        st = _lib.load().gr_volproj(ctypes.byref(atoms.struct), dim, ctypes.cast(n, ctypes.c_void_p),
                                    ctypes.cast(ptrs, ctypes.c_void_p), u.data_ptr(),
                                    engine._stream_handle(dev))
    _lib.check(st, "gr_volproj")
    return u


def volproj_into(atoms, y, u, dim, psf=False):
    """VolProj(atom, y, u): write the rendering into u (host array or tensor)."""
    out = volproj(atoms, y, psf=psf)
    if isinstance(u, torch.Tensor):
        u.copy_(out.reshape(u.shape))
    else:
        u[...] = out.cpu().numpy().reshape(np.shape(u))
