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
