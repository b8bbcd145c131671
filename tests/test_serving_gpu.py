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
    # the finished fits' loop graphs wait for close(), not for the results
    assert srv._retired_loops
    srv.close()
    assert not srv._retired_loops
    assert all(res[i]["admitted"] <= res[i]["finish"] for i in res)


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


def test_lean_plain_loop_gives_the_same_fits(cuda_ready):
    """The plain loop without the reference structure's repeated work (no
    re-projection of the current atoms, no derivatives after a rejection)
    takes exactly the same steps."""
    ref = serving.serve_plain(_requests(n=4))
    lean = serving.serve_plain(_requests(n=4), lean=True)
    for k in ref:
        assert ref[k]["iterations"] == lean[k]["iterations"]
        assert ref[k]["loss"] == lean[k]["loss"]
        assert ref[k]["accepted"] == lean[k]["accepted"]


def test_admission_failure_waits_for_memory_then_runs(cuda_ready):
    """An allocation failure at admission (injected on the host: the hook
    raises the allocator's out-of-memory error once) puts the request back at
    the head of the queue; it is admitted again once a fit has finished and
    its result equals the undisturbed one.  With nothing in flight, a request
    that cannot be allocated ends with an error result and the server goes
    on."""
    reqs = _requests(n=4)
    for r in reqs:
        r.arrival = 0.0
    clean_srv = serving.GaussFitServer(max_slots=4, n_streams=4)
    for r in _requests(n=4):
        r.arrival = 0.0
        clean_srv.submit(r)
    clean = clean_srv.run()
    srv = serving.GaussFitServer(max_slots=4, n_streams=4)
    fired, calls = [], []

    def fault(req):
        # the second admission: one fit is then in flight
        calls.append(req.id)
        if len(calls) == 2 and not fired:
            fired.append(req.id)
            raise torch.cuda.OutOfMemoryError("injected: no memory for this request now")
    srv._admit_fault = fault
    for r in reqs:
        srv.submit(r)
    res = srv.run()
    assert fired and srv.admission_retries == 1
    for k in clean:
        assert res[k]["status"] == clean[k]["status"]
        assert np.array_equal(res[k]["theta"], clean[k]["theta"])
    # nothing in flight: the request cannot ever fit -> error, others still run
    srv2 = serving.GaussFitServer(max_slots=1, n_streams=1)
    reqs2 = _requests(n=2)

    def always(req):
        if req.id == reqs2[0].id:
            raise torch.cuda.OutOfMemoryError("injected")
    srv2._admit_fault = always
    for r in reqs2:
        r.arrival = 0.0
        srv2.submit(r)
    res2 = srv2.run()
    assert res2[reqs2[0].id]["status"] == "error"
    assert res2[reqs2[1].id]["status"] in ("ok", "no_progress")


def test_cancel_queued_and_in_flight_requests(cuda_ready):
    """cancel(): a queued request leaves the queue; one in flight finishes
    its device work, then its result is discarded.  The others are not
    affected."""
    reqs = _requests(n=5)
    for r in reqs:
        r.arrival = 0.0
    srv = serving.GaussFitServer(max_slots=2, n_streams=2)
    for r in reqs:
        srv.submit(r)
    assert srv.cancel(reqs[4].id)             # still queued
    srv._admit(0.0)                            # two fits now in flight
    inflight = srv.active[0].req.id
    assert srv.cancel(inflight)
    assert not srv.cancel(12345)
    res = srv.run()
    assert res[reqs[4].id]["status"] == "cancelled"
    assert res[inflight]["status"] == "cancelled"
    clean_srv = serving.GaussFitServer(max_slots=2, n_streams=2)
    for r in _requests(n=5):
        r.arrival = 0.0
        clean_srv.submit(r)
    clean = clean_srv.run()
    for k in res:
        if res[k]["status"] != "cancelled":
            assert np.array_equal(res[k]["theta"], clean[k]["theta"])
    assert not srv.active and srv.in_use == 0


def test_tuned_server_runs_each_class_under_its_plans(cuda_ready):
    """tune_request_classes times candidate schedules per shape class under
    plans; a tuned server's fits match the untuned ones (the schedule only
    changes FP rounding of derivative chunk sums)."""
    tuning = importlib.import_module(PKG + ".tuning")
    reqs = _requests(n=4)
    n = tuning.tune_request_classes(reqs, torch.device("cuda"), reps=1)
    assert n >= 1
    assert all(p is not None for p in tuning.plans_for_request(reqs[0]))
    srv = serving.GaussFitServer(max_slots=4, n_streams=4, tuned=True)
    base = serving.GaussFitServer(max_slots=4, n_streams=4)
    for r, q in zip(reqs, _requests(n=4)):
        r.arrival = q.arrival = 0.0
        srv.submit(r)
        base.submit(q)
    a, b = srv.run(), base.run()
    for k in a:
        assert abs(a[k]["loss"] - b[k]["loss"]) <= 1e-4 * abs(b[k]["loss"])
        assert a[k]["loss"] <= a[k]["loss0"]


def test_regularised_served_fit_matches_plain_fit(cuda_ready):
    """A request with a regulariser (the reference's Newton loop takes one:
    NewtonGaussian.py:59-66): its value joins the loss and its gradient and
    Hessian the blocks, in the device loop as in the plain loop."""
    regm = importlib.import_module(PKG + ".regularisation")

    def reqs():
        out = _requests(n=4)
        for r in out:
            r.arrival = 0.0
            dim = len(r.init[1][0])
            r.reg = regm.Joubert(dim, 1e-3, 1e-2, (1e-3, 1e-4))
        return out
    srv = serving.GaussFitServer(max_slots=4, n_streams=2)
    for r in reqs():
        srv.submit(r)
    served = srv.run()
    srv.close()
    plain = serving.serve_plain(reqs())
    bare = serving.serve_plain(_requests(n=4))
    for k in plain:
        # the same trajectory: the same accepted steps and trials, the same loss
        assert served[k]["accepted"] == plain[k]["accepted"]
        assert abs(served[k]["loss"] - plain[k]["loss"]) <= 1e-12 * abs(plain[k]["loss"])
        # the regulariser changed the fit
        assert served[k]["loss"] != bare[k]["loss"]


def _small_2d(n=8, seed=21):
    return workloads.config3_requests(n=n, rate=1e9, seed=seed, p2d=1.0, atoms=(8, 150),
                                      angles=(10, 40), det=(24, 96), max_iter=40, tol=1e-6)


def test_batched_small_fits_equal_their_own_loops(cuda_ready):
    """Small 2D fits admitted together run as one batched device loop
    (engine.BatchLoop: each kernel one launch over the batch's table of
    problems); every fit ends exactly where its own device loop ends."""
    def run(batch_max):
        srv = serving.GaussFitServer(max_slots=16, n_streams=4, batch_max=batch_max)
        for r in _small_2d():
            r.arrival = 0.0
            srv.submit(r)
        res = srv.run()
        srv.close()
        return srv, res
    s1, own = run(1)
    s8, batched = run(32)
    assert s1.batches == 0 and s8.batches >= 1
    assert set(own) == set(batched)
    for k in own:
        a, b = own[k], batched[k]
        assert a["iterations"] == b["iterations"] and a["accepted"] == b["accepted"]
        assert np.array_equal(a["theta"], b["theta"])
        assert a["loss"] == b["loss"] and a["loss0"] == b["loss0"]


def test_batch_members_alone_equal_members_in_a_batch(cuda_ready):
    """A batchable fit alone (a batch of one) and among others: the same."""
    alone = {}
    for r in _small_2d(n=5, seed=22):
        r.arrival = 0.0
        srv = serving.GaussFitServer(max_slots=1, n_streams=1, batch_max=8)
        srv.submit(r)
        alone.update(srv.run())
        srv.close()
    srv = serving.GaussFitServer(max_slots=8, n_streams=2, batch_max=8)
    for r in _small_2d(n=5, seed=22):
        r.arrival = 0.0
        srv.submit(r)
    mix = srv.run()
    srv.close()
    assert srv.batches >= 1
    for k in alone:
        assert np.array_equal(alone[k]["theta"], mix[k]["theta"])
        assert alone[k]["iterations"] == mix[k]["iterations"]


def test_skipping_empty_items_leaves_served_fits_unchanged(cuda_ready):
    """3D fits whose forwards skip the items no atom meets end bitwise where
    the fits with full forwards end (same iterations, parameters, loss)."""
    def reqs():
        return workloads.config3_requests(n=4, rate=1e9, seed=12, p2d=0.0, atoms=(6, 40),
                                          angles=(10, 30), det=(64, 128), max_iter=30, tol=1e-6)
    out = {}
    for skip in (True, False):
        srv = serving.GaussFitServer(max_slots=4, n_streams=2, skip_empty=skip)
        for r in reqs():
            r.arrival = 0.0
            srv.submit(r)
        out[skip] = srv.run()
        srv.close()
    assert set(out[True]) == set(out[False])
    for k in out[True]:
        a, b = out[True][k], out[False][k]
        assert a["iterations"] == b["iterations"]
        assert np.array_equal(a["theta"], b["theta"])
        assert a["loss"] == b["loss"]
