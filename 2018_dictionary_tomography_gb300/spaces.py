"""Atom, projection and volume spaces of the dictionary API, without ODL.

Mirrors GaussDictCode/dictionary_def.py: AtomSpace (:72), AtomElement (:147),
VolSpace (:217), ProjSpace (:261), ProjElement (:338).  Attribute names,
array layouts and error behaviour follow the reference:

* AtomElement holds ``x`` (N, dim), ``r`` (N, 1) isotropic or (N, dim(dim+1)/2)
  packed upper-triangular, ``I`` (N,), float32 host arrays by default (the
  reference casts through its context's fType, float32 in every demo);
* ProjSpace is built from angle partitions (``angles``, ``detector``) or from
  explicit ``orientations`` / ``ortho`` frames, and exposes ``orientations``
  (A, d), ``ortho`` (tuple of (A, d)), ``detector`` (list of 1-D cell-centre
  arrays) and ``shape``.

Partitions are anything with ``grid.coord_vectors`` or ``coord_vectors`` (an
ODL partition works), or plain arrays; :func:`uniform_partition` builds one.
"""
import numpy as np

from .geometry import perp, theta_to_vec

DTYPE = np.float32


class Partition:
    """Minimal uniform partition: cell centres per axis (``coord_vectors``)."""

    def __init__(self, coord_vectors, min_pt, max_pt):
        self.coord_vectors = tuple(np.asarray(c, dtype=np.float64) for c in coord_vectors)
        self.min_pt = np.atleast_1d(np.asarray(min_pt, dtype=np.float64))
        self.max_pt = np.atleast_1d(np.asarray(max_pt, dtype=np.float64))
        self.shape = tuple(c.size for c in self.coord_vectors)

    @property
    def grid(self):
        return self

    @property
    def ndim(self):
        return len(self.coord_vectors)


def uniform_partition(min_pt, max_pt, shape, nodes_on_bdry=False):
    """Cell centres of a uniform partition (odl.uniform_partition semantics:
    with nodes_on_bdry the first/last nodes sit on the boundary)."""
    min_pt = np.atleast_1d(np.asarray(min_pt, dtype=np.float64))
    max_pt = np.atleast_1d(np.asarray(max_pt, dtype=np.float64))
    shape = np.atleast_1d(shape).astype(int)
    if min_pt.size == 1 and shape.size > 1:
        min_pt = np.repeat(min_pt, shape.size)
        max_pt = np.repeat(max_pt, shape.size)
    cv = []
    for lo, hi, n in zip(min_pt, max_pt, shape):
        if nodes_on_bdry:
            cv.append(np.linspace(lo, hi, n) if n > 1 else np.array([0.5 * (lo + hi)]))
        else:
            h = (hi - lo) / n
            cv.append(lo + h * (np.arange(n) + 0.5))
    return Partition(cv, min_pt, max_pt)


def _getcoord_vectors(thing):
    """Coordinate vectors of a partition-like object (dictionary_def.py:395)."""
    if hasattr(thing, "grid") and hasattr(thing.grid, "coord_vectors"):
        return tuple(np.asarray(c) for c in thing.grid.coord_vectors)
    if hasattr(thing, "coord_vectors"):
        return tuple(np.asarray(c) for c in thing.coord_vectors)
    if hasattr(thing, "__getitem__"):
        if np.isscalar(thing[0]):
            return (np.asarray(thing),)
        return tuple(np.asarray(t) for t in thing)
    raise ValueError("could not read coordinate vectors")


def _host(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


class AtomSpace:
    """Space of Gaussian atoms of dimension ``dim`` (dictionary_def.py:72)."""

    def __init__(self, dim, isotropic=True):
        self.dim = dim
        self.isotropic = isotropic
        self._size = 1 + dim + (1 if isotropic else (3 if dim == 2 else 6))

    @property
    def n_params(self):
        return self._size

    def element(self, *args, **kwargs):
        if len(args) == 1:
            arr = np.asarray(args[0])
            if arr.ndim == 2 and arr.shape[1] == self._size:
                return AtomElement(self, arr[:, 1:self.dim + 1], arr[:, self.dim + 1:],
                                   arr[:, :1], **kwargs)
            raise ValueError("input could not be interpetted")
        return AtomElement(self, *args, **kwargs)

    def zero(self):
        return AtomElement(self, np.zeros((0, self.dim)), np.zeros(0), np.zeros(0))

    empty = zero

    def random(self, n, seed=None):
        """Random atoms as AtomSpace.random (dictionary_def.py:130-139)."""
        if seed is not None:
            np.random.seed(seed)
        if self.isotropic:
            r = np.random.rand(n, 1) + 1
        else:
            r = np.random.rand(n, (self.dim * (self.dim + 1)) // 2) + 1
            r[:, self.dim:] /= 4
        return AtomElement(self, .8 * (2 * np.random.rand(n, self.dim) - 1), r,
                           2 * np.random.rand(n))

    def copy(self):
        return AtomSpace(self.dim, self.isotropic)

    def __eq__(self, other):
        return (self.dim == getattr(other, "dim", None)
                and self.isotropic == getattr(other, "isotropic", None))

    def __hash__(self):
        return hash((self.dim, self.isotropic))


class AtomElement:
    """A set of atoms (I, x, r) (dictionary_def.py:147-214)."""

    def __init__(self, space, x=None, r=None, I=None):
        self.space = space
        x = np.array(_host(x), dtype=np.float64, copy=True)
        r = np.array(_host(r), dtype=np.float64, copy=True)
        I = np.array(_host(I), dtype=np.float64, copy=True)
        d = space.dim
        pr = (d * (d + 1)) // 2
        self.x = x.reshape(-1, d)
        n = self.x.shape[0]
        if r.size == 1:
            if space.isotropic:
                r = r * np.ones(n)
            else:
                r = r * np.ones((n, pr))
                r[:, d:] = 0
        elif (not space.isotropic) and (r.size == n):
            r = np.tile(r.reshape(-1, 1), pr)
            r[:, d:] = 0
        self.r = r.reshape(n, -1)
        if space.isotropic:
            if self.r.size != n:
                raise ValueError("isotropic atoms take one radius each")
        elif 2 * self.r.shape[1] != d * (d + 1):
            raise ValueError("anisotropic atoms take %d radius entries each" % pr)
        if I.size == 1:
            I = I * np.ones(n)
        self.I = I.reshape(-1)
        if self.I.size != n:
            raise ValueError("one intensity per atom")
        self.x = self.x.astype(DTYPE)
        self.r = self.r.astype(DTYPE)
        self.I = self.I.astype(DTYPE)
        self.size = self.I.size

    def copy(self):
        return AtomElement(self.space, self.x, self.r, self.I)

    def __getitem__(self, i):
        if np.isscalar(i):
            i = slice(i, i + 1) if i >= 0 else slice(i, i + 1 if i != -1 else None)
        return AtomElement(self.space, self.x[i], self.r[i], self.I[i])

    def __setitem__(self, i, atoms):
        if np.isscalar(i):
            i = slice(i, i + 1)
        self.x[i] = atoms.x
        self.r[i] = atoms.r
        self.I[i] = atoms.I
        return self

    @property
    def data(self):
        n = self.x.shape[0]
        return np.concatenate([self.I.reshape(n, 1), self.x, self.r.reshape(n, -1)], axis=1)

    def asarray(self):
        return self.data

    def __len__(self):
        return self.size


class VolSpace:
    """Voxel grid of the embedding (dictionary_def.py:217-232)."""

    def __init__(self, partition):
        self.partition = partition
        self.coord_vectors = tuple(np.asarray(c, dtype=DTYPE) for c in _getcoord_vectors(partition))
        self.shape = tuple(c.size for c in self.coord_vectors)

    def element(self, arr):
        return VolElement(self, arr)


class VolElement:
    def __init__(self, space, u):
        self.space = space
        u = _host(u) if not _is_cuda(u) else u
        if np.isscalar(u) or getattr(u, "size", None) == 1:
            u = u * np.ones(space.shape, dtype=DTYPE)
        self.data = u

    def asarray(self):
        return self.data

    def copy(self):
        return VolElement(self.space, self.data.copy())


def _is_cuda(a):
    try:
        import torch
        return isinstance(a, torch.Tensor) and a.is_cuda
    except ImportError:
        return False


class ProjSpace:
    """Projection (sinogram) space (dictionary_def.py:261-335)."""

    def __init__(self, angles=None, detector=None, orientations=None, ortho=None):
        if angles is not None:
            angles = _getcoord_vectors(angles)
            self.orientations = theta_to_vec(angles)
            self.ortho = perp(angles)
        elif orientations is not None and ortho is not None:
            self.orientations = _host(orientations)
            self.ortho = tuple(_host(o) for o in ortho)
        else:
            raise ValueError("give angles, or orientations and ortho")
        dim = self.orientations.shape[-1]
        self.orientations = np.asarray(self.orientations, dtype=DTYPE).reshape(-1, dim)
        self.ortho = tuple(np.asarray(o, dtype=DTYPE).reshape(-1, dim) for o in self.ortho)
        self.detector = [np.asarray(g, dtype=DTYPE).reshape(-1) for g in _getcoord_vectors(detector)]
        self.shape = [self.orientations.shape[0]] + [g.size for g in self.detector]

    @property
    def dim(self):
        d = self.orientations.shape[1]
        return 3 if (d == 3 or len(self.detector) == 2) else 2

    def element(self, arr=None):
        return ProjElement(self, 0 if arr is None else arr)

    def zero(self):
        return ProjElement(self, 0)

    def one(self):
        return ProjElement(self, 1)

    def random(self):
        return ProjElement(self, np.random.rand(*self.shape))

    def copy(self):
        return ProjSpace(orientations=self.orientations.copy(),
                         ortho=tuple(o.copy() for o in self.ortho),
                         detector=tuple(g.copy() for g in self.detector))

    def __getitem__(self, sl):
        return ProjSpace(orientations=self.orientations[sl],
                         ortho=tuple(o[sl] for o in self.ortho), detector=self.detector)

    def __eq__(self, other):
        shape = getattr(other, "shape", [None])
        return len(shape) == len(self.shape) and all(a == b for a, b in zip(shape, self.shape))

    def __hash__(self):
        return id(self)

    @property
    def volume(self):
        return self.orientations.shape[0] * abs(np.prod([p[-1] + p[1] - 2 * p[0]
                                                          for p in self.detector]))


class ProjElement:
    """A sinogram (dictionary_def.py:338-371); data is a host array or a CUDA
    tensor of shape ``space.shape``."""

    def __init__(self, space, u):
        self.space = space
        if _is_cuda(u):
            data = u
        else:
            u = _host(u)
            if np.isscalar(u) or u.size == 1:
                u = u * np.ones(space.shape)
            data = np.asarray(u, dtype=DTYPE)
        if tuple(data.shape) != tuple(space.shape):
            raise ValueError("Shape of array does not match shape of space")
        self.data = data
        self.shape = tuple(data.shape)

    def asarray(self):
        return self.data

    def copy(self):
        return ProjElement(self.space, self.data.clone() if _is_cuda(self.data) else self.data.copy())

    def _other(self, o):
        return o.data if isinstance(o, ProjElement) else o

    def __add__(self, o):
        return ProjElement(self.space, self.data + self._other(o))

    def __sub__(self, o):
        return ProjElement(self.space, self.data - self._other(o))

    def __mul__(self, o):
        return ProjElement(self.space, self.data * self._other(o))

    __rmul__ = __mul__

    def __neg__(self):
        return ProjElement(self.space, -self.data)
