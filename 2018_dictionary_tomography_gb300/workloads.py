"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations.  The reference's real datasets are not available;
these generators stand in for them.

All generators return plain numpy arrays (float64) in the reference layout:
atoms (I (N,), x (N, d), r (N, P_r) upper-triangular packed, or (N, 1)
isotropic) and a geometry (orientations, ortho tuple, detector tuple).
A "lower-triangular covariance factor T" of a configuration is stored as the
reference's upper-triangular r = T^T (same diagonal, same off-diagonal
distribution), packed [r00 r11 r01] (2D) or [r00 r11 r22 r01 r12 r02] (3D).
"""
import numpy as np

from .geometry import perp, theta_to_vec


class Workload:
    def __init__(self, name, truth, init, orientations, ortho, detector, data,
                 fit="l2", background=0.0, extra=None):
        self.name = name
        self.truth = truth          # (I, x, r)
        self.init = init            # (I, x, r)
        self.orientations = orientations
        self.ortho = ortho
        self.detector = detector
        self.data = data
        self.fit = fit
        self.background = background
        self.extra = extra or {}

    @property
    def shape(self):
        return (self.orientations.shape[0],) + tuple(len(d) for d in self.detector)


def cell_centres(lo, hi, n):
    """Cell centres of a uniform partition of [lo, hi] into n cells."""
    h = (hi - lo) / n
    return lo + h * (np.arange(n) + 0.5)


def angle_nodes(lo, hi, n):
    """Angles of a uniform partition with nodes on the boundary
    (odl.uniform_partition(lo, hi, n, nodes_on_bdry=True))."""
    if n == 1:
        return np.array([0.5 * (lo + hi)])
    return np.linspace(lo, hi, n)


def aniso_r(rng, n, dim, diag, off_sd):
    pr = 3 if dim == 2 else 6
    r = np.empty((n, pr))
    r[:, :dim] = rng.uniform(diag[0], diag[1], (n, dim))
    r[:, dim:] = rng.normal(0.0, off_sd, (n, pr - dim))
    return r


def project_host(I, x, r, orientations, ortho, detector):
    """Forward projection on the GPU engine, returned to the host."""
    import torch
    from . import engine
    from .geometry import DeviceGeometry
    g = DeviceGeometry(orientations, ortho, detector)
    R = engine.radproj(engine.DeviceAtoms(I, x, r), g)
    torch.cuda.synchronize()
    return R.cpu().numpy().astype(np.float64)


def config0(seed=0, project=project_host):
    """2D isotropic GD fit: 64 atoms, 60 angles on [0, pi), 128 cells on
    [-1.5, 1.5]; std U[0.02, 0.08] -> r = 1/(sqrt(60) std); data noise
    N(0, (0.01 max)^2); init jitters centres N(0, 0.03), I x U[0.7, 1.3]."""
    rng = np.random.default_rng(seed)
    N = 64
    x = rng.uniform(-0.6, 0.6, (N, 2))
    I = rng.uniform(0.5, 1.5, N)
    sd = rng.uniform(0.02, 0.08, N)
    r = (1.0 / (np.sqrt(60.0) * sd)).reshape(N, 1)
    th = np.linspace(0, np.pi, 60, endpoint=False)
    T = theta_to_vec([th])
    w = perp([th])
    det = (cell_centres(-1.5, 1.5, 128),)
    clean = project(I, x, r, T, w, det)
    data = clean + rng.normal(0.0, 0.01 * clean.max(), clean.shape)
    init = (I * rng.uniform(0.7, 1.3, N), x + rng.normal(0, 0.03, x.shape), r.copy())
    return Workload("config0: 2D iso GD, 64 atoms, 60x128", (I, x, r), init, T, w, det,
                    data, "l2", extra={"iters": 200})


def config1(seed=1, project=project_host, peak_photons=1e4, background=1.0):
    """2D anisotropic Newton fit with KL loss: 512 atoms, factor diag U[8, 40],
    off-diagonal N(0, 5); 180 angles on [0, pi); 256 cells on [-1.5, 1.5];
    Poisson counts scaled to a peak of 1e4 photons plus a background."""
    rng = np.random.default_rng(seed)
    N = 512
    x = rng.uniform(-0.6, 0.6, (N, 2))
    I = rng.uniform(0.5, 1.5, N)
    r = aniso_r(rng, N, 2, (8.0, 40.0), 5.0)
    th = np.linspace(0, np.pi, 180, endpoint=False)
    T = theta_to_vec([th])
    w = perp([th])
    det = (cell_centres(-1.5, 1.5, 256),)
    clean = project(I, x, r, T, w, det)
    scale = peak_photons / clean.max()
    I = I * scale
    counts = rng.poisson(clean * scale + background).astype(np.float64)
    init = (I * rng.uniform(0.7, 1.3, N), x + rng.normal(0, 0.01, x.shape), r.copy())
    return Workload("config1: 2D aniso KL Newton, 512 atoms, 180x256", (I, x, r), init,
                    T, w, det, counts, "kl", background, extra={"iters": 30})


def config2(seed=2, project=project_host):
    """3D single-axis tilt: 4096 atoms in [-1, 1]^3, factor diag U[10, 50],
    off-diagonal N(0, 6), I U[0.2, 2]; 121 tilts on [-60, 60] degrees about the
    tilt axis (atom coordinate 2, the reference's 2.5D geometry); 256 x 256
    cells on [-1.5, 1.5]^2; L2 loss."""
    rng = np.random.default_rng(seed)
    N = 4096
    x = rng.uniform(-1.0, 1.0, (N, 3))
    I = rng.uniform(0.2, 2.0, N)
    r = aniso_r(rng, N, 3, (10.0, 50.0), 6.0)
    th = angle_nodes(-np.pi / 3, np.pi / 3, 121)
    T = theta_to_vec([th])
    w = perp([th])
    c = cell_centres(-1.5, 1.5, 256)
    det = (c, c.copy())
    data = None
    if project is not None:
        clean = project(I, x, r, T, w, det)
        data = clean + rng.normal(0.0, 0.01 * clean.max(), clean.shape)
    init = (I * rng.uniform(0.9, 1.1, N), x + rng.normal(0, 0.005, x.shape), r.copy())
    return Workload("config2: 3D tilt series, 4096 atoms, 121x256x256", (I, x, r), init,
                    T, w, det, data, "l2")


def random_rotations(rng, n):
    """Uniform random rotations (unit quaternions)."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    a, b, c, d = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = a * a + b * b - c * c - d * d
    R[:, 0, 1] = 2 * (b * c - a * d)
    R[:, 0, 2] = 2 * (b * d + a * c)
    R[:, 1, 0] = 2 * (b * c + a * d)
    R[:, 1, 1] = a * a - b * b + c * c - d * d
    R[:, 1, 2] = 2 * (c * d - a * b)
    R[:, 2, 0] = 2 * (b * d - a * c)
    R[:, 2, 1] = 2 * (c * d + a * b)
    R[:, 2, 2] = a * a - b * b - c * c + d * d
    return R


def config4(seed=4, n_orient=20000, project=project_host, snr=0.1):
    """Single-particle style: 8192 atoms (as config 2) at n_orient orientations
    uniform on SO(3) given as explicit frames (T, w0, w1 = columns of a random
    rotation); 128 x 128 cells on [-1, 1]^2; per-image Gaussian noise at the
    given SNR (signal power / noise power)."""
    rng = np.random.default_rng(seed)
    N = 8192
    x = rng.uniform(-0.7, 0.7, (N, 3))
    I = rng.uniform(0.2, 2.0, N)
    r = aniso_r(rng, N, 3, (10.0, 50.0), 6.0)
    R = random_rotations(rng, n_orient)
    w0, w1, T = R[:, :, 0], R[:, :, 1], R[:, :, 2]
    c = cell_centres(-1.0, 1.0, 128)
    det = (c, c.copy())
    data = None
    if project is not None:
        clean = project(I, x, r, T, (w0, w1), det)
        p = np.mean(clean.reshape(n_orient, -1) ** 2, axis=1)
        sd = np.sqrt(p / snr)
        data = clean + rng.normal(size=clean.shape) * sd[:, None, None]
    init = (I * rng.uniform(0.9, 1.1, N), x + rng.normal(0, 0.005, x.shape), r.copy())
    return Workload("config4: single-particle, 8192 atoms, %d x 128x128" % n_orient,
                    (I, x, r), init, T, (w0, w1), det, data, "l2")


def config3_requests(n=512, rate=200.0, seed=3, p2d=0.6, atoms=(16, 4096),
                     angles=(30, 180), det=(64, 512), max_iter=100, tol=1e-6):
    """Served stream: n fitting requests with Poisson arrivals at ``rate``/s;
    each 2D (probability p2d, isotropic atoms as config 0) or 3D (single-axis
    tilt series, anisotropic atoms as config 2); atom count log-uniform in
    ``atoms``, angle count uniform in ``angles``, detector cells per side
    uniform in ``det``; data = projection + N(0, (0.01 max)^2) with a
    per-request seed; init = truth with jittered centres and intensities;
    L2 Newton to relative loss change ``tol`` (at most ``max_iter``)."""
    from .serving import FitRequest
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for i in range(n):
        rr = np.random.default_rng([seed, i])
        is2d = rr.uniform() < p2d
        N = int(round(np.exp(rr.uniform(np.log(atoms[0]), np.log(atoms[1])))))
        A = int(rr.integers(angles[0], angles[1] + 1))
        D = int(rr.integers(det[0], det[1] + 1))
        if is2d:
            x = rr.uniform(-0.6, 0.6, (N, 2))
            I = rr.uniform(0.5, 1.5, N)
            sd = rr.uniform(0.02, 0.08, N)
            r = (1.0 / (np.sqrt(60.0) * sd)).reshape(N, 1)
            th = np.linspace(0, np.pi, A, endpoint=False)
            T, w = theta_to_vec([th]), perp([th])
            detc = (cell_centres(-1.5, 1.5, D),)
            jit = 0.1 * sd.reshape(N, 1)
        else:
            x = rr.uniform(-1.0, 1.0, (N, 3))
            I = rr.uniform(0.2, 2.0, N)
            r = aniso_r(rr, N, 3, (10.0, 50.0), 6.0)
            th = angle_nodes(-np.pi / 3, np.pi / 3, A)
            T, w = theta_to_vec([th]), perp([th])
            c = cell_centres(-1.5, 1.5, D)
            detc = (c, c.copy())
            jit = 0.1 / (np.sqrt(60.0) * r[:, :3].max(axis=1, keepdims=True))
        init = (I * rr.uniform(0.9, 1.1, N), x + rr.normal(0, 1, x.shape) * jit, r.copy())
        truth = (I, x, r)
        reqs.append(FitRequest(i, T, w, detc, init, _data_maker(truth, [seed, i]), "l2", 0.0,
                               max_iter=max_iter, tol=tol, arrival=float(t[i])))
    return reqs


def materialize_data(requests, device):
    """Generate every request's data sinogram once (on the device, as
    ``make_data`` does) and keep it in pinned host memory as
    ``req.data_host``: the request then carries its payload, and admission
    only copies it to the device."""
    import torch
    from .geometry import DeviceGeometry
    for req in requests:
        geom = DeviceGeometry(req.orientations, req.ortho, req.detector, device)
        d = req.make_data(geom, device, torch.cuda.current_stream(device))
        req.data_host = d.cpu().pin_memory()
    torch.cuda.synchronize(device)
    return requests


def _data_maker(truth, seed):
    def make(geom, device, stream):
        import torch
        from . import engine
        R = engine.radproj(engine.DeviceAtoms(*truth, device), geom)
        gen = torch.Generator(device=device)
        gen.manual_seed(int(np.random.default_rng(seed).integers(1 << 62)))
        noise = torch.randn(R.shape, generator=gen, device=device, dtype=torch.float32)
        return (R + noise * (0.01 * R.max())).contiguous()
    return make
