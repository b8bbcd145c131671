"""A CPU stand-in for the parts of ``numba`` the reference's kernel modules use.

TEST INFRASTRUCTURE ONLY: used by ``make_ref_golden.py`` to run the reference's
own Numba-CUDA source (GaussDictCode/bin/{numba_cuda_aux,NewtonBases,
NewtonBases2D,point_spread_functions}.py) on the CPU of this container, where
numba is not installed, so that golden vectors come from the reference's code
rather than from a restatement of it.

What it emulates (the only ``numba`` API those files touch):

* ``cuda.jit(device=True)`` -> the plain Python function (device functions);
  ``cuda.jit`` / ``cuda.jit(...)`` without ``device`` -> a kernel object that is
  launched as ``kernel[grid, block](*args)``;
* the SIMT launch: every thread of every block runs the kernel body, with
  ``cuda.threadIdx``, ``cuda.blockIdx``, ``cuda.blockDim``, ``cuda.gridDim``
  and ``cuda.grid(n)`` per thread.  Kernels that declare shared memory run the
  threads of one block as Python threads that meet at ``cuda.syncthreads()``
  (a ``threading.Barrier``), so the reference's shared-memory tree reductions
  (numba_cuda_aux.py:135-179) execute exactly as written; other kernels run
  their threads one after another;
* ``cuda.local.array`` -> a fresh zeroed numpy array per call;
  ``cuda.shared.array`` -> one array per block, the k-th declaration of every
  thread of a block returning the same array;
* ``numba.jit`` -> identity; ``float32``/``int32`` -> numpy dtypes.

Precision: ``PRECISION`` (numpy float64 by default) is the dtype that
``float32`` maps to, so the reference's arithmetic runs in FP64 and its results
pin an FP64 oracle to ~1e-13.  ``math.exp``/``math.sqrt`` (the reference's
``c_exp``/``c_sqrt``) are CPython's.
"""
import sys
import threading
import types

import numpy as np

PRECISION = np.float64

_tls = threading.local()


class _Dim3:
    __slots__ = ("x", "y", "z")

    def __init__(self, v):
        v = tuple(v) + (1,) * (3 - len(v))
        self.x, self.y, self.z = int(v[0]), int(v[1]), int(v[2])


def _as3(v):
    return (int(v), 1, 1) if np.isscalar(v) else tuple(int(a) for a in v) + (1,) * (3 - len(v))


class _dtype_marker:
    def __init__(self, name):
        self.name = name


float32 = _dtype_marker("f4")
int32 = _dtype_marker("i4")


def _np_dtype(dt):
    if isinstance(dt, _dtype_marker):
        return PRECISION if dt.name == "f4" else np.int32
    if dt in ("f4", "float32"):
        return PRECISION
    return dt


class _Local:
    @staticmethod
    def array(shape, dtype):
        return np.zeros(shape, dtype=_np_dtype(dtype))


class _Shared:
    @staticmethod
    def array(shape, dtype):
        st = _tls.state
        k = _tls.shared_calls
        _tls.shared_calls += 1
        with st["lock"]:
            arrs = st["shared"]
            while len(arrs) <= k:
                arrs.append(None)
            if arrs[k] is None:
                arrs[k] = np.zeros(shape, dtype=_np_dtype(dtype))
            return arrs[k]


class _Idx:
    def __init__(self, attr):
        self._attr = attr

    def __getattr__(self, name):
        return getattr(getattr(_tls, self._attr), name)


class _Kernel:
    def __init__(self, fn):
        self.fn = fn
        try:
            import inspect
            src = inspect.getsource(fn)
        except (OSError, TypeError):
            src = ""
        self.uses_shared = "shared.array" in src or "syncthreads" in src

    def __call__(self, *args):
        return self.fn(*args)

    def __getitem__(self, cfg):
        grid, block = _as3(cfg[0]), _as3(cfg[1])
        return lambda *args: _launch(self, grid, block, args)


def _thread_body(kern, args, bidx, tidx, grid, block, state, errors):
    _tls.threadIdx = _Dim3(tidx)
    _tls.blockIdx = _Dim3(bidx)
    _tls.blockDim = _Dim3(block)
    _tls.gridDim = _Dim3(grid)
    _tls.state = state
    _tls.shared_calls = 0
    try:
        kern.fn(*args)
    except threading.BrokenBarrierError:
        pass
    except BaseException as e:  # noqa: BLE001 - re-raised by the launcher
        errors.append(e)
        if state.get("barrier") is not None:
            state["barrier"].abort()


def _launch(kern, grid, block, args):
    nthr = block[0] * block[1] * block[2]
    errors = []
    for bz in range(grid[2]):
        for by in range(grid[1]):
            for bx in range(grid[0]):
                state = {"lock": threading.Lock(), "shared": [], "barrier": None}
                tids = [(tx, ty, tz) for tz in range(block[2]) for ty in range(block[1])
                        for tx in range(block[0])]
                if kern.uses_shared and nthr > 1:
                    state["barrier"] = threading.Barrier(nthr)
                    ths = [threading.Thread(target=_thread_body,
                                            args=(kern, args, (bx, by, bz), t, grid, block,
                                                  state, errors)) for t in tids]
                    for t in ths:
                        t.start()
                    for t in ths:
                        t.join()
                else:
                    for t in tids:
                        _thread_body(kern, args, (bx, by, bz), t, grid, block, state, errors)
                if errors:
                    raise errors[0]


def _syncthreads():
    b = _tls.state.get("barrier")
    if b is not None:
        b.wait()


def _grid(n):
    t, b, d = _tls.threadIdx, _tls.blockIdx, _tls.blockDim
    g = (b.x * d.x + t.x, b.y * d.y + t.y, b.z * d.z + t.z)
    return g[0] if n == 1 else g[:n]


def jit(*args, **kw):
    if len(args) == 1 and callable(args[0]) and not kw:
        return _Kernel(args[0])
    device = kw.get("device", False)

    def deco(fn):
        return fn if device else _Kernel(fn)
    return deco


def _host_jit(*args, **kw):
    if len(args) == 1 and callable(args[0]) and not kw:
        return args[0]
    return lambda fn: fn


def install():
    """Put a ``numba`` package (with ``numba.cuda``) into sys.modules."""
    numba = types.ModuleType("numba")
    cuda = types.ModuleType("numba.cuda")
    cuda.jit = jit
    cuda.local = _Local
    cuda.shared = _Shared
    cuda.syncthreads = _syncthreads
    cuda.grid = _grid
    cuda.threadIdx = _Idx("threadIdx")
    cuda.blockIdx = _Idx("blockIdx")
    cuda.blockDim = _Idx("blockDim")
    cuda.gridDim = _Idx("gridDim")
    numba.cuda = cuda
    numba.jit = _host_jit
    numba.float32 = float32
    numba.int32 = int32
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda
    return numba
