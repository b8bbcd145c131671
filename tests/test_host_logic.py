"""Host-side logic of the serving path and the fit-step graph, on the CPU:
arena layouts and views, the memory estimate used for admission, and the
seeded served-stream generator."""
import importlib

import numpy as np
import pytest
import torch

PKG = "2018_dictionary_tomography_gb300"
serving = importlib.import_module(PKG + ".serving")
engine = importlib.import_module(PKG + ".engine")
workloads = importlib.import_module(PKG + ".workloads")


def _items():
    return [("theta", np.float64, (37, 10)), ("flags", np.uint8, (5,)),
            ("counter", np.int32, (1,)), ("empty", np.float32, (0, 4)),
            ("field", np.float32, (3, 17, 19)), ("scalar", np.float64, ())]


def test_layout_is_aligned_disjoint_and_sized():
    spec, total = serving._layout(_items())
    ends = []
    for name, dt, shape in _items():
        off, sdt, sshape, nb = spec[name]
        assert off % serving._ALIGN == 0, name
        assert sdt == np.dtype(dt) and sshape == tuple(shape)
        assert nb == int(np.prod(shape, dtype=np.int64)) * np.dtype(dt).itemsize
        ends.append((off, off + nb))
    ends.sort()
    for (a0, a1), (b0, _b1) in zip(ends, ends[1:]):
        assert a1 <= b0
    assert total >= ends[-1][1] and total % serving._ALIGN == 0
    # an empty request still gets a non-empty arena
    assert serving._layout([])[1] == serving._ALIGN


def test_device_and_host_views_agree_and_do_not_alias():
    spec, total = serving._layout(_items())
    buf = torch.zeros(total, dtype=torch.uint8)
    arr = buf.numpy()                       # the same memory, seen from numpy
    rng = np.random.default_rng(0)
    view = serving._typed_views(buf)
    for name, dt, shape in _items():
        v = view(spec[name])
        assert tuple(v.shape) == tuple(shape)
        vals = rng.integers(0, 100, size=shape).astype(dt)
        v.copy_(torch.from_numpy(np.array(vals)))  # keeps 0-d shapes
    # every buffer still holds its own values (no view overlaps another)
    rng = np.random.default_rng(0)
    for name, dt, shape in _items():
        vals = rng.integers(0, 100, size=shape).astype(dt)
        assert np.array_equal(serving._host_view(arr, spec[name]), vals), name
        assert np.array_equal(view(spec[name]).numpy(), vals), name


def test_fit_step_packing_is_aligned_and_disjoint():
    items = [("I", (7,)), ("x", (7, 3)), ("r", (7, 6)), ("data", (5, 11, 13)), ("loss", ())]
    spec, total = engine._pack(items)
    buf = torch.zeros(total, dtype=torch.float64)
    for k, (name, shape) in enumerate(items):
        off, sshape = spec[name]
        assert off % 64 == 0 and tuple(sshape) == tuple(shape)
        engine._packed_view(buf, spec[name]).fill_(k + 1)
    for k, (name, shape) in enumerate(items):
        assert bool((engine._packed_view(buf, spec[name]) == k + 1).all()), name


def test_memory_estimate_grows_with_the_problem():
    reqs = workloads.config3_requests(n=40, seed=5)
    est = [(serving.GaussFitServer.estimate_bytes(r), r) for r in reqs]
    assert all(b > 0 for b, _ in est)
    # the estimate covers at least the request's fit fields and data (float32)
    for b, r in est:
        assert b >= 3 * 4 * r.size_hint[1]
    # more cells, same atoms: a larger estimate
    r = reqs[0]
    small = serving.GaussFitServer.estimate_bytes(r)
    n, cells = r.size_hint
    r.size_hint = (n, 4 * cells)
    try:
        assert serving.GaussFitServer.estimate_bytes(r) > small
    finally:
        r.size_hint = (n, cells)


def test_served_stream_is_seeded_and_within_its_ranges():
    a = workloads.config3_requests(n=64, seed=9)
    b = workloads.config3_requests(n=64, seed=9)
    c = workloads.config3_requests(n=64, seed=10)
    arr = [r.arrival for r in a]
    assert arr == sorted(arr) and arr[0] > 0
    assert arr == [r.arrival for r in b]
    assert arr != [r.arrival for r in c]
    dims = []
    for ra, rb in zip(a, b):
        n, cells = ra.size_hint
        assert (n, cells) == rb.size_hint
        for xa, xb in zip(ra.init, rb.init):
            assert np.array_equal(xa, xb)
        dim = len(ra.init[1][0])
        dims.append(dim)
        assert 16 <= n <= 4096
        A = len(ra.orientations)
        assert 30 <= A <= 180
        D = len(ra.detector[0])
        assert 64 <= D <= 512
        assert cells == A * D ** (dim - 1)
        assert ra.fit == "l2" and ra.max_iter == 100
    assert set(dims) == {2, 3}


def _valid_request():
    wl = importlib.import_module(PKG + ".workloads")
    return wl.config3_requests(n=1, seed=5, atoms=(8, 16), angles=(10, 12), det=(24, 32))[0]


def test_malformed_requests_are_refused_before_the_device():
    """validate_request (GaussFitServer.submit): shape mismatches, NaN
    parameters or data, empty atom sets and bad fit settings raise ValueError
    on the host."""
    import copy

    import torch
    serving = importlib.import_module(PKG + ".serving")
    req = _valid_request()
    serving.validate_request(req)
    cases = []
    r = copy.copy(req)
    I, x, rr = req.init
    r.init = (I[:0], x[:0], rr[:0])
    cases.append(("no atoms", r))
    r = copy.copy(req)
    r.init = (I, x[:, :1], rr)
    cases.append(("x shape", r))
    r = copy.copy(req)
    x2 = np.array(x, dtype=np.float64)
    x2[0, 0] = np.nan
    r.init = (I, x2, rr)
    cases.append(("nan atom", r))
    r = copy.copy(req)
    r.ortho = (np.asarray(req.ortho[0])[:-1],)
    cases.append(("ortho length", r))
    r = copy.copy(req)
    r.orientations = np.zeros((0, 2))
    cases.append(("no angles", r))
    r = copy.copy(req)
    r.fit, r.background = "kl", 0.0
    cases.append(("kl background", r))
    r = copy.copy(req)
    r.max_iter = 0
    cases.append(("max_iter", r))
    r = copy.copy(req)
    r.reg = "joubert"
    cases.append(("regulariser object", r))
    r = copy.copy(req)
    regm = importlib.import_module(PKG + ".regularisation")
    r.reg = regm.Joubert(len(req.init[1][0]), float("nan"), 1e-2, (1e-3, 1e-4))
    cases.append(("regulariser parameters", r))
    r = copy.copy(req)
    shape = (len(req.orientations),) + tuple(len(d) for d in req.detector)
    bad = torch.zeros(shape)
    bad[0].view(-1)[0] = float("inf")
    r.data_host = bad
    cases.append(("inf data", r))
    r = copy.copy(req)
    r.data_host = torch.zeros(3, 3)
    cases.append(("data shape", r))
    for what, rq in cases:
        with pytest.raises(ValueError):
            serving.validate_request(rq)


def test_angle_range_views_the_parent_geometry():
    """DeviceGeometry.angle_range: a sub-geometry over the parent's buffers
    (frame records offset by a0 records, same detector), no copy."""
    geometry = importlib.import_module(PKG + ".geometry")
    th = np.linspace(0, np.pi, 12, endpoint=False)
    T = np.stack([-np.sin(th), np.cos(th)], 1)
    w = np.stack([np.cos(th), np.sin(th)], 1)
    g = geometry.DeviceGeometry(T, (w,), (np.linspace(-1, 1, 40),), device="cpu")
    sub = g.angle_range(3, 9)
    assert sub.n_angles == 6 and sub.shape == (6, 40)
    assert sub.struct.n_angles == 6 and sub.struct.kdet == g.struct.kdet
    stride = g.frames.shape[1] * g.frames.element_size()
    assert sub.struct.frames == g.struct.frames + 3 * stride
    assert sub.struct.det[0] == g.struct.det[0]
    assert np.array_equal(sub.frames.numpy(), g.frames.numpy()[3:9])
    with pytest.raises(ValueError):
        g.angle_range(5, 13)


def test_when_idle_admission_promotes_the_largest_arrived_request():
    """Under-loaded (fewer fits in flight than half the streams): the largest
    arrived request goes first; loaded: arrival order is kept; requests that
    have not arrived are never promoted."""
    import collections
    import types
    serving = importlib.import_module(PKG + ".serving")
    R = lambda rid, arr, n, cells: types.SimpleNamespace(id=rid, arrival=arr,
                                                         size_hint=(n, cells))
    reqs = [R(0, 0.0, 16, 100), R(1, 0.0, 900, 5000), R(2, 0.1, 4000, 9000),
            R(3, 0.0, 900, 5000), R(4, 0.0, 30, 40)]
    pend = collections.deque(reqs)
    got = serving.promote_when_idle(pend, now=0.05, n_active=3, n_streams=31)
    # request 2 has not arrived; 1 and 3 tie, the earlier wins
    assert got.id == 1 and [r.id for r in pend] == [1, 0, 2, 3, 4]
    pend.popleft()
    assert serving.promote_when_idle(pend, now=0.2, n_active=0, n_streams=31).id == 2
    assert [r.id for r in pend] == [2, 0, 3, 4]
    # loaded: nothing moves
    assert serving.promote_when_idle(pend, now=0.2, n_active=15, n_streams=31) is None
    assert [r.id for r in pend] == [2, 0, 3, 4]
    # nothing arrived yet
    late = collections.deque([R(7, 1.0, 50, 50)])
    assert serving.promote_when_idle(late, now=0.0, n_active=0, n_streams=31) is None
