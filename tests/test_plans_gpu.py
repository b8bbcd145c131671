"""Per-plan schedules (gr_plan): two streams running different work splits
and tilings at the same time give exactly what each gives alone.  The
process-wide schedule stays untouched."""
import importlib

import numpy as np
import pytest
import torch

from problems import engine_atoms, engine_geometry, make_atoms, make_geometry

pytestmark = pytest.mark.gpu
PKG = "2018_dictionary_tomography_gb300"


def _problem(seed):
    g = make_geometry("3d", 36, 72, 80)
    I, x, r = make_atoms(3, 600, seed, rdiag=(4.0, 12.0), roff=1.5, box=0.7)
    data = np.random.default_rng(seed).normal(size=g.shape).astype(np.float32)
    return engine_geometry(g), engine_atoms(I, x, r), torch.from_numpy(data).cuda()


def _fit(eng, geom, atoms, data, plan_p, plan_d, order):
    fw = eng.fit_forward(atoms, geom, data, "l2", 0.0, want_R=True, plan=plan_p)
    f, g, H = eng.atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, order, plan=plan_d)
    return [fw["R"], fw["loss"], g] + ([H] if H is not None else [])


def test_concurrent_streams_with_different_plans(eng, cuda_ready):
    lib = importlib.import_module(PKG + "._lib")
    ga, aa, da = _problem(1)
    gb, ab, db = _problem(2)
    saved = [lib.load().gr_get_tuning(k) for k in (0, 1, 2, 3, 4, 6, 7)]
    pa_p = eng.Plan(lib.GR_OP_PROJECT, aa, ga).set(3, 1).set(4, 0)
    pa_d = eng.Plan(lib.GR_OP_DERIVS_2, aa, ga).set(7, 0).set(0, 8192).set(1, 2)
    pb_p = eng.Plan(lib.GR_OP_PROJECT, ab, gb).set(3, 2).set(4, 1 << 30)
    pb_d = eng.Plan(lib.GR_OP_DERIVS_2, ab, gb).set(7, 1024).set(6, 0)
    alone_a = [t.clone() for t in _fit(eng, ga, aa, da, pa_p, pa_d, 2)]
    alone_b = [t.clone() for t in _fit(eng, gb, ab, db, pb_p, pb_d, 2)]
    torch.cuda.synchronize()
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(3):
        with torch.cuda.stream(sa):
            ra = _fit(eng, ga, aa, da, pa_p, pa_d, 2)
        with torch.cuda.stream(sb):
            rb = _fit(eng, gb, ab, db, pb_p, pb_d, 2)
        torch.cuda.synchronize()
        for x, y in zip(ra + rb, alone_a + alone_b):
            assert torch.equal(x, y)
    # the plans did not touch the process-wide schedule
    assert [lib.load().gr_get_tuning(k) for k in (0, 1, 2, 3, 4, 6, 7)] == saved
    # the tiling leaves the projection bitwise equal (cells sum their atoms in
    # index order): plan b's 32 x 32 tiles against the default 16 x 32 ones,
    # both with the block split of small problems
    rd = _fit(eng, gb, ab, db, None, None, 2)
    assert torch.equal(rd[0], alone_b[0])


def test_autotuned_plan_per_shape_class(eng, cuda_ready):
    lib = importlib.import_module(PKG + "._lib")
    tuning = importlib.import_module(PKG + ".tuning")
    geom, atoms, data = _problem(3)
    fw = eng.fit_forward(atoms, geom, data, "l2", 0.0)
    saved = [lib.load().gr_get_tuning(k) for k in (0, 1, 2)]
    best = tuning.autotune_derivs(atoms, geom, fw["alpha"], None, 1.0, order=1, reps=2,
                                  candidates=[(4096, 1, 1), (131072, 1, 1), (16384, 2, 2)])
    assert best is not None
    plan = tuning.plan_for(atoms, geom, 1)
    assert plan is not None and tuning.apply_for(atoms, geom, 1) == best[:3]
    assert [lib.load().gr_get_tuning(k) for k in (0, 1, 2)] == saved
    f, g, _ = eng.atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, 1, plan=plan)
    f0, g0, _ = eng.atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, 1)
    scale = g0.abs().amax(0).clamp_min(1e-30)
    assert float(((g - g0).abs() / scale).max()) < 1e-5


@pytest.mark.parametrize("fit", ["l2", "kl"])
@pytest.mark.parametrize("form,split", [(1, 0), (1, 1 << 30), (2, 0), (2, 1 << 30)])
def test_forward_skipping_empty_items(eng, cuda_ready, fit, form, split):
    """The 3D forward that skips the items no atom meets (their loss from a
    record of the data alone) gives bitwise the loss of the full forward,
    and its fields wherever an atom is, under both tilings, with and without
    the block split of small problems; the derivatives from its fields are
    bitwise those from the full forward's."""
    lib = importlib.import_module(PKG + "._lib")
    g = make_geometry("2p5d", 24, 96, 80)
    I, x, r = make_atoms(3, 40, 5, rdiag=(8.0, 20.0), roff=1.5, box=0.3)
    geom, atoms = engine_geometry(g), engine_atoms(I, x, r)
    rng = np.random.default_rng(6)
    data = torch.from_numpy(rng.uniform(0.5, 2.0, size=g.shape).astype(np.float32)).cuda()
    bg = 0.5 if fit == "kl" else 0.0
    plan = eng.Plan(lib.GR_OP_PROJECT, atoms, geom).set(3, form).set(4, split)
    full = eng.fit_forward(atoms, geom, data, fit, bg, want_R=True, plan=plan)
    n_items = eng.fit_items(geom, plan)
    assert n_items == g.shape[0] * ((96 + (16 if form == 1 else 32) - 1) //
                                    (16 if form == 1 else 32)) * ((80 + 31) // 32)
    ws, _ = eng._ws_for(lib.GR_OP_PROJECT, atoms, geom, plan)
    empty = torch.empty(n_items, dtype=torch.float64, device="cuda")
    eng.fit_empty_loss_into(atoms, geom, data, fit, bg, empty, ws, plan=plan)
    alpha = torch.full(g.shape, float("nan"), dtype=torch.float32, device="cuda")
    beta = torch.full(g.shape, float("nan"), dtype=torch.float32, device="cuda") \
        if fit == "kl" else None
    loss = torch.empty((), dtype=torch.float64, device="cuda")
    eng.fit_forward_into(atoms, geom, data, fit, bg, None, alpha, beta, loss, ws, plan=plan,
                         empty_loss=empty)
    torch.cuda.synchronize()
    assert loss.item() == full["loss"].item()
    written = ~torch.isnan(alpha)
    # the atoms meet part of the detector only: items were skipped
    assert 0.02 < written.float().mean().item() < 0.95
    assert written[full["R"] != 0].all()
    assert torch.equal(alpha[written], full["alpha"][written])
    if fit == "kl":
        assert torch.equal(beta[written], full["beta"][written])
    # the derivatives read the fields inside the atoms' supports only
    d_full = eng.atom_derivs(atoms, geom, "field", full["alpha"], full["beta"],
                             1.0 if fit == "l2" else 0.0, 2)
    d_skip = eng.atom_derivs(atoms, geom, "field", alpha, beta, 1.0 if fit == "l2" else 0.0, 2)
    for a, b in zip(d_full, d_skip):
        assert torch.equal(a, b)


def test_forward_skipping_rejects_2d_and_R(eng, cuda_ready):
    lib = importlib.import_module(PKG + "._lib")
    g = make_geometry("2d", 12, 64)
    I, x, r = make_atoms(2, 10, 1)
    geom, atoms = engine_geometry(g), engine_atoms(I, x, r)
    assert eng.fit_items(geom) == 0
    data = torch.zeros(g.shape, dtype=torch.float32, device="cuda")
    ws, _ = eng._ws_for(lib.GR_OP_PROJECT, atoms, geom)
    out = torch.empty(8, dtype=torch.float64, device="cuda")
    with pytest.raises(lib.EngineError):
        eng.fit_empty_loss_into(atoms, geom, data, "l2", 0.0, out, ws)
    loss = torch.empty((), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        eng.fit_forward_into(atoms, geom, data, "l2", 0.0, data.clone(), None, None, loss, ws,
                             empty_loss=out)
