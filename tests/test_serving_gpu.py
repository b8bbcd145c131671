"""Continuous-batching server: each result is the same alone and in the mix;
admission by a memory budget; requests admitted while others run."""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"
serving = importlib.import_module(PKG + ".serving")
workloads = importlib.import_module(PKG + ".workloads")


def _requests(n=6, rate=1e9):
    # small mixed stream: 2D and 3D, uneven sizes
    return workloads.config3_requests(n=n, rate=rate, seed=11, atoms=(8, 96), angles=(10, 40),
                                      det=(24, 64), max_iter=40, tol=1e-6)


def test_results_alone_equal_results_in_the_mix(cuda_ready):
    alone = {}
    for req in _requests():
        req.arrival = 0.0
        srv = serving.GaussFitServer(max_slots=1, n_streams=1)
        srv.submit(req)
        alone.update(srv.run())
    mix_srv = serving.GaussFitServer(max_slots=8, n_streams=4)
    for req in _requests():
        req.arrival = 0.0
        mix_srv.submit(req)
    mix = mix_srv.run()
    assert set(mix) == set(alone)
    for k in alone:
        a, b = alone[k], mix[k]
        assert a["iterations"] == b["iterations"]
        assert np.allclose(a["theta"], b["theta"], rtol=1e-6, atol=0)
        assert abs(a["loss"] - b["loss"]) <= 1e-6 * abs(a["loss"])
        # the kernels are deterministic and the state private: in fact bitwise
        assert np.array_equal(a["theta"], b["theta"])


def test_admission_by_memory_budget_and_while_busy(cuda_ready):
    reqs = _requests(n=8)
    for i, r in enumerate(reqs):
        r.arrival = 0.002 * i
    ests = sorted(serving.GaussFitServer.estimate_bytes(r) for r in reqs)
    budget = ests[-1] + ests[-2]          # the two largest fit, not all eight
    assert sum(ests) > budget
    srv = serving.GaussFitServer(max_slots=8, n_streams=4, hbm_budget=budget)
    peak, peak_bytes = [0], [0]
    orig = srv._admit

    def admit(now):
        orig(now)
        peak[0] = max(peak[0], len(srv.active))
        peak_bytes[0] = max(peak_bytes[0], srv.in_use)
    srv._admit = admit
    for r in reqs:
        srv.submit(r)
    res = srv.run()
    assert len(res) == 8
    assert peak_bytes[0] <= budget
    assert peak[0] < 8
    assert srv.admitted_while_busy > 0


def test_served_fit_matches_plain_fit(cuda_ready):
    reqs = _requests(n=3)
    for r in reqs:
        r.arrival = 0.0
    srv = serving.GaussFitServer(max_slots=4, n_streams=2, iters_per_launch=1)
    for r in reqs:
        srv.submit(r)
    served = srv.run()
    plain = serving.serve_plain(_requests(n=3))
    for k in plain:
        # same update rule; the served loop checks convergence after each
        # iteration here, so both stop at the same iteration
        assert abs(served[k]["loss"] - plain[k]["loss"]) <= 1e-5 * abs(plain[k]["loss"])


def test_device_loop_matches_host_stepped_graphs(cuda_ready):
    """The device-resident loop (one graph launch per fit, stop test on the
    device) and the host-stepped one-iteration graphs (stop test on the host
    after every iteration) apply the same rule: same iterations, bitwise
    the same parameters."""
    reqs = _requests(n=4)
    for r in reqs:
        r.arrival = 0.0
    dev_srv = serving.GaussFitServer(max_slots=4, n_streams=2)
    for r in reqs:
        dev_srv.submit(r)
    dev = dev_srv.run()
    assert dev_srv.device_loops == len(reqs)
    host_srv = serving.GaussFitServer(max_slots=4, n_streams=2, device_loop=False,
                                      iters_per_launch=1)
    reqs2 = _requests(n=4)
    for r in reqs2:
        r.arrival = 0.0
        host_srv.submit(r)
    host = host_srv.run()
    assert host_srv.device_loops == 0
    for k in dev:
        assert dev[k]["iterations"] == host[k]["iterations"]
        assert np.array_equal(dev[k]["theta"], host[k]["theta"])


def test_gated_derivatives_match_eager_loop_after_rejections(cuda_ready):
    """In the device loop the derivative launches sit in an IF node that
    skips them after a rejected trial (the atoms did not move).  On a fit
    that rejects trials, the result equals bit for bit the eager loop, which
    evaluates the derivatives at every iteration."""
    dev = torch.device("cuda")
    reqs = workloads.config3_requests(n=48, seed=3)
    # a 2D request of 40 atoms that rejects about a quarter of its trials
    req = [r for r in reqs if len(r.init[1][0]) == 2 and r.size_hint[0] == 40][0]
    workloads.materialize_data([req], dev)
    srv = serving.GaussFitServer(dev, max_slots=2, n_streams=1)
    st = srv.streams[0]
    s = serving._Slot(req, st, dev, True, 4, True, srv.setup_stream)
    assert s.loop is not None
    with torch.cuda.stream(st):
        s.launch()
    torch.cuda.synchronize()
    gated = s.result()
    acc = s.h_acc.numpy()[:gated["iterations"]]
    assert (acc == 0).any() and (acc == 1).any()
    e = serving._Slot(req, st, dev, False, 1, False, srv.setup_stream)
    assert e.loop is None
    while True:
        torch.cuda.synchronize()
        if e.done():
            break
        e.launch()
    eager = e.result()
    assert gated["iterations"] == eager["iterations"]
    assert np.array_equal(gated["theta"], eager["theta"])
    assert gated["loss"] == eager["loss"]
    s.loop.close()
