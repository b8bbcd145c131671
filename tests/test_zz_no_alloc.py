"""gr_radproj_noalloc: the forward projection for callers that cannot
allocate device memory (a host that owns the GPU memory budget, a binding
without a device allocator, a loop that must not call cudaMalloc).

It is called here through the C ABI exactly as such a caller would: device
pointers in, nothing allocated by the library.  Its output must match the
workspace-taking gr_radproj on two calls in a row, with different problems,
so a leftover scratch from the first call cannot leak into the second.
The file name sorts last so a failure here stops a -x run only after every
other test has run; the test also passes alone in a fresh process.
"""
import ctypes
import importlib

import numpy as np
import pytest
import torch

from problems import engine_atoms, engine_geometry, make_atoms, make_geometry

pytestmark = pytest.mark.gpu

TOL = 1e-5
GR_ERR_TOO_LARGE = -5


def _raw_lib():
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib_mod.load()  # builds the library if needed
    raw = ctypes.CDLL(lib_mod.library_path())
    P = ctypes.POINTER
    raw.gr_radproj_noalloc.restype = ctypes.c_int
    raw.gr_radproj_noalloc.argtypes = [P(lib_mod.GrAtoms), P(lib_mod.GrGeometry),
                                       ctypes.c_void_p, ctypes.c_void_p]
    raw.gr_radproj.restype = ctypes.c_int
    raw.gr_radproj.argtypes = [P(lib_mod.GrAtoms), P(lib_mod.GrGeometry), ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    raw.gr_workspace_bytes.restype = ctypes.c_size_t
    raw.gr_workspace_bytes.argtypes = [ctypes.c_int, P(lib_mod.GrAtoms), P(lib_mod.GrGeometry)]
    return raw


def _reference_projection(raw, atoms, geom, stream):
    """gr_radproj with a caller-allocated workspace."""
    n = raw.gr_workspace_bytes(0, ctypes.byref(atoms.struct), ctypes.byref(geom.struct))
    ws = torch.empty(max(n, 256), dtype=torch.uint8, device="cuda")
    out = torch.full(geom.shape, -7.0, dtype=torch.float32, device="cuda")
    rc = raw.gr_radproj(ctypes.byref(atoms.struct), ctypes.byref(geom.struct),
                        out.data_ptr(), ws.data_ptr(), n, stream)
    assert rc == 0
    return out


def test_noalloc_projection_matches_gr_radproj_twice(cuda_ready):
    raw = _raw_lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    problems = [
        (make_geometry("3d", 9, 40, 44), make_atoms(3, 12, 21)),
        (make_geometry("2d", 30, 96), make_atoms(2, 40, 22)),
    ]
    for g, (I, x, r) in problems:
        atoms, geom = engine_atoms(I, x, r), engine_geometry(g)
        ref = _reference_projection(raw, atoms, geom, stream)
        out = torch.full(geom.shape, 123.0, dtype=torch.float32, device="cuda")
        rc = raw.gr_radproj_noalloc(ctypes.byref(atoms.struct), ctypes.byref(geom.struct),
                                    out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.max(np.abs(a - b)) <= TOL * np.max(np.abs(b))


def test_noalloc_rejects_problems_beyond_its_scratch(cuda_ready):
    raw = _raw_lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # 3D, 4096 atoms, 200 angles of 256 x 256 cells: bitmaps far above 4 MiB
    g = make_geometry("2p5d", 200, 256, 256)
    I, x, r = make_atoms(3, 4096, 23)
    atoms, geom = engine_atoms(I, x, r), engine_geometry(g)
    need = raw.gr_workspace_bytes(0, ctypes.byref(atoms.struct), ctypes.byref(geom.struct))
    assert need > (4 << 20)
    out = torch.zeros(geom.shape, dtype=torch.float32, device="cuda")
    rc = raw.gr_radproj_noalloc(ctypes.byref(atoms.struct), ctypes.byref(geom.struct),
                                out.data_ptr(), stream)
    assert rc == GR_ERR_TOO_LARGE
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0
