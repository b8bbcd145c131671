"""Projection geometry: ray directions, detector frames and detector grids.

``theta_to_vec`` / ``perp`` restate GaussDictCode/atomFuncs.py:13-74 (ray
direction T and detector axes for one angle vector in 2D, two in 3D).
``DeviceGeometry`` turns a ProjSpace's (orientations, ortho, detector) into the
per-angle frame records the CUDA engine reads (include/gauss_radon.h).
"""
import numpy as np
import torch

from . import _lib


def theta_to_vec(theta):
    """Ray directions: 2D (-sin t, cos t); 3D (-sin t0 cos t1, cos t0 cos t1,
    sin t1) on the grid of the two angle vectors (atomFuncs.py:13-47)."""
    theta = [np.asarray(t, dtype=np.float64).reshape(-1) for t in theta]
    if len(theta) == 1:
        t = theta[0]
        return np.stack([-np.sin(t), np.cos(t)], axis=-1)
    if len(theta) == 2:
        t0, t1 = np.meshgrid(theta[0], theta[1], indexing="ij")
        return np.stack([-np.sin(t0) * np.cos(t1), np.cos(t0) * np.cos(t1),
                         np.sin(t1)], axis=-1)
    raise ValueError("theta_to_vec takes one (2D) or two (3D) angle vectors")


def perp(theta):
    """Detector axes orthogonal to theta_to_vec (atomFuncs.py:50-74)."""
    theta = [np.asarray(t, dtype=np.float64).reshape(-1) for t in theta]
    if len(theta) == 1:
        t = theta[0]
        return (np.stack([np.cos(t), np.sin(t)], axis=-1),)
    if len(theta) == 2:
        t0, t1 = np.meshgrid(theta[0], theta[1], indexing="ij")
        o0 = np.stack([np.cos(t0), np.sin(t0), np.zeros_like(t0)], axis=-1)
        o1 = np.stack([np.sin(t0) * np.sin(t1), -np.cos(t0) * np.sin(t1),
                       np.cos(t1)], axis=-1)
        return o0, o1
    raise ValueError("perp takes one (2D) or two (3D) angle vectors")


def _np(a):
    if isinstance(a, torch.Tensor):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def uniform_grid(coords, name="detector"):
    """(first, inverse step) of an increasing, uniformly spaced grid."""
    c = np.asarray(coords, dtype=np.float64).reshape(-1)
    if c.size == 1:
        return float(c[0]), 1.0
    d = np.diff(c)
    step = (c[-1] - c[0]) / (c.size - 1)
    if not step > 0:
        raise ValueError("%s coordinates must be increasing" % name)
    if np.max(np.abs(d - step)) > 1e-4 * abs(step):
        raise ValueError("%s coordinates must be uniformly spaced" % name)
    return float(c[0]), float(1.0 / step)


def frame_records(orientations, ortho, n_det_axes):
    """Frame records (FP32) and kdet from reference-layout arrays: T, the
    detector axes, and the first kdet rows of inverse([w0 (w1) T]) as an FP32
    pair (rounded rows, then their residues), 8 (2D) or 24 (3D) floats.

    orientations (A, 2|3); ortho tuple of (A, 2|3); n_det_axes 1 or 2.
    2D: T, w0 of length 2, one detector axis.  2.5D (reference
    NewtonBases.py:685-688): T, w0 of length 2 with two detector axes, the
    second along atom coordinate 2.  3D: T, w0, w1 of length 3.
    """
    T = np.asarray(_np(orientations), dtype=np.float32).astype(np.float64)
    T = T.reshape(-1, T.shape[-1])
    w = [np.asarray(_np(o), dtype=np.float32).astype(np.float64).reshape(T.shape[0], -1)
         for o in ortho]
    A, dT = T.shape
    if dT == 2 and n_det_axes == 1:
        kdet, stride = 1, 8
        B = np.stack([w[0], T], axis=2)               # (A, 2, 2) columns w0, T
        cols = [w[0], T]
    elif dT == 2 and n_det_axes == 2:
        kdet, stride = 2, 24
        z = np.zeros((A, 1))
        T3 = np.concatenate([T, z], axis=1)
        w03 = np.concatenate([w[0], z], axis=1)
        w13 = np.tile(np.array([[0.0, 0.0, 1.0]]), (A, 1))
        cols = [w03, w13, T3]
        B = np.stack(cols[:2] + [T3], axis=2)
    elif dT == 3 and n_det_axes == 2 and len(w) >= 2:
        kdet, stride = 2, 24
        cols = [w[0], w[1], T]
        B = np.stack(cols, axis=2)
    else:
        raise ValueError("unsupported geometry: orientation dim %d with %d detector axes"
                         % (dT, n_det_axes))
    det = np.linalg.det(B)
    if np.any(np.abs(det) < 1e-8):
        raise ValueError("detector axes and ray direction must be linearly independent")
    Binv = np.linalg.inv(B)                           # rows: dual basis
    D = kdet + 1
    rec = np.zeros((A, stride), dtype=np.float64)
    rec[:, 0:D] = cols[-1]
    for k in range(kdet):
        rec[:, D * (1 + k):D * (2 + k)] = cols[k]
    # dual rows as an FP32 pair hi + lo (the kernels form the projection
    # centre B^{-1} x from both)
    hi = Binv.astype(np.float32).astype(np.float64)
    lo = Binv - hi
    for k in range(kdet):
        rec[:, D * (1 + kdet + k):D * (2 + kdet + k)] = hi[:, k, :]
        rec[:, D * (1 + 2 * kdet + k):D * (2 + 2 * kdet + k)] = lo[:, k, :]
    return rec.astype(np.float32), kdet


class DeviceGeometry:
    """Geometry resident in device memory, plus the C-ABI descriptor."""

    def __init__(self, orientations, ortho, detector, device=None):
        device = torch.device(device or "cuda")
        detector, rec, kdet = self.host_records(orientations, ortho, detector)
        frames = torch.from_numpy(rec).to(device)
        det = [torch.from_numpy(d.copy()).to(device) for d in detector]
        self._bind(rec, kdet, detector, frames, det, device)

    @staticmethod
    def host_records(orientations, ortho, detector):
        """(detector coordinate arrays, frame records, kdet) on the host."""
        detector = [np.asarray(_np(d), dtype=np.float32).reshape(-1) for d in detector]
        rec, kdet = frame_records(orientations, ortho, len(detector))
        if len(detector) != kdet:
            raise ValueError("detector must have %d coordinate vectors" % kdet)
        return detector, rec, kdet

    @classmethod
    def bound(cls, rec, kdet, detector, frames, det, device):
        """A geometry over device buffers that hold (or will hold, by a copy
        queued before any use) the frame records ``rec`` and the detector
        coordinates: no allocation, no copy."""
        self = cls.__new__(cls)
        self._bind(rec, kdet, detector, frames, det, torch.device(device))
        return self

    def _bind(self, rec, kdet, detector, frames, det, device):
        self.kdet = kdet
        self.dim = kdet + 1
        self.n_angles = rec.shape[0]
        self.frames_host = rec
        self.frames = frames
        self.det = det
        self.grid = [uniform_grid(d, "detector axis %d" % k) for k, d in enumerate(detector)]
        self.shape = (self.n_angles,) + tuple(int(d.size) for d in detector)
        self.device = device
        s = _lib.GrGeometry()
        s.kdet = kdet
        s.n_angles = self.n_angles
        s.frames = self.frames.data_ptr()
        for k in range(2):
            if k < kdet:
                s.n_det[k] = int(self.det[k].numel())
                s.det[k] = self.det[k].data_ptr()
                s.det_first[k] = self.grid[k][0]
                s.det_inv_step[k] = self.grid[k][1]
            else:
                s.n_det[k] = 1
                s.det[k] = None
                s.det_first[k] = 0.0
                s.det_inv_step[k] = 1.0
        self.struct = s

    def angle_range(self, a0, a1):
        """The geometry of angles [a0, a1) over this one's device buffers
        (no allocation, no copy): rows a0..a1-1 of a sinogram on this
        geometry are a sinogram on it."""
        if not 0 <= a0 < a1 <= self.n_angles:
            raise ValueError("angle range [%d, %d) outside [0, %d)" % (a0, a1, self.n_angles))
        sub = DeviceGeometry.__new__(DeviceGeometry)
        sub.kdet, sub.dim = self.kdet, self.dim
        sub.n_angles = a1 - a0
        sub.frames_host = self.frames_host[a0:a1]
        sub.frames = self.frames[a0:a1]
        sub.det, sub.grid, sub.device = self.det, self.grid, self.device
        sub.shape = (a1 - a0,) + tuple(self.shape[1:])
        st = _lib.GrGeometry.from_buffer_copy(self.struct)
        st.n_angles = sub.n_angles
        st.frames = sub.frames.data_ptr()
        sub.struct = st
        return sub

    @staticmethod
    def from_space(space, device=None):
        """From an object with .orientations, .ortho, .detector (ProjSpace)."""
        return DeviceGeometry(space.orientations, space.ortho, space.detector, device)
