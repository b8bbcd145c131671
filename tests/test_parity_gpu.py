"""GPU parity of the CUDA engine against the FP64 oracle.

Tolerance for the FP32 path: 1e-5 relative (sinograms and losses normwise;
gradients and Hessians per parameter entry, scaled by that entry's largest
magnitude over the atoms)."""
import numpy as np
import pytest
import torch

from oracle import gauss_oracle as go
from problems import (engine_atoms, engine_geometry, entry_relerr, make_atoms,
                      make_geometry, relerr)

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = {
    "2d": dict(kind="2d", A=30, D0=96, N=24, dim=2),
    "2p5d": dict(kind="2p5d", A=9, D0=40, D1=36, N=10, dim=3),
    "3d": dict(kind="3d", A=9, D0=40, D1=44, N=10, dim=3),
}


def _setup(case, iso=False, seed=0):
    c = CASES[case]
    g = make_geometry(c["kind"], c["A"], c["D0"], c.get("D1"))
    I, x, r = make_atoms(c["dim"], c["N"], seed, iso=iso)
    return g, I, x, r


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("iso", [False, True])
def test_forward_matches_oracle(eng, cuda_ready, case, iso):
    g, I, x, r = _setup(case, iso)
    R = eng.radproj(engine_atoms(I, x, r), engine_geometry(g)).cpu().numpy()
    ref = go.radproj(I, x, r, g)
    assert R.shape == ref.shape
    assert relerr(R, ref) < TOL


def test_forward_large_2d_matches_oracle(eng, cuda_ready):
    """Config-0 sized 2D problem (64 atoms, 60 angles, 128 cells)."""
    g = make_geometry("2d", 60, 128)
    I, x, r = make_atoms(2, 64, 11, iso=True, rdiag=(1.61, 6.45), box=0.6)
    R = eng.radproj(engine_atoms(I, x, r), engine_geometry(g)).cpu().numpy()
    assert relerr(R, go.radproj(I, x, r, g)) < TOL


def test_forward_and_kl_fit_many_2d_atoms(eng, cuda_ready):
    """1100 atoms: tiles' atom lists span >= 32 bitmap words, so eight warps
    share each 2D tile (the long-list form of the 2D projection)."""
    g = make_geometry("2d", 24, 160)
    I, x, r = make_atoms(2, 1100, 13, box=0.6)
    geom, atoms = engine_geometry(g), engine_atoms(I, x, r)
    Ro = go.radproj(I, x, r, g)
    R = eng.radproj(atoms, geom).cpu().numpy()
    assert relerr(R, Ro) < TOL
    counts = np.random.default_rng(4).poisson(Ro + 1.0).astype(np.float64)
    fw = eng.fit_forward(atoms, geom, torch.from_numpy(counts).float().cuda(), "kl", 1.0)
    lo = go.kl_value(counts, Ro, 1.0)
    assert abs(fw["loss"].item() - lo) <= TOL * abs(lo)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("order", [1, 2])
def test_inner_derivs_match_oracle(eng, cuda_ready, case, order):
    g, I, x, r = _setup(case, seed=1)
    C = np.random.default_rng(2).normal(size=g.shape).astype(np.float32).astype(np.float64)
    f, gr_, H = eng.atom_derivs(engine_atoms(I, x, r), engine_geometry(g), "inner",
                                torch.from_numpy(C).float(), order=order)
    fo, go_, Ho = go.all_atom_derivs("ip", I, x, r, g, C, 2)
    assert relerr(f.cpu().numpy(), fo) < TOL
    assert entry_relerr(gr_.cpu().numpy(), go_) < TOL
    if order == 2:
        assert entry_relerr(H.cpu().numpy(), Ho) < TOL


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("iso", [False, True])
def test_l2_fit_derivs_match_oracle(eng, cuda_ready, case, iso):
    """All-atom L2 derivatives = reference L2derivs_RadProj(atom_j,
    data + R_j - R) for every j (NewtonGaussian.py:59-60)."""
    g, I, x, r = _setup(case, iso=iso, seed=3)
    rng = np.random.default_rng(4)
    data = (go.radproj(I * 0.9, x + 0.01, r, g) + rng.normal(0, 0.01, g.shape))
    data = data.astype(np.float32).astype(np.float64)
    loss, gr_, H = eng.l2_fit_derivs(engine_atoms(I, x, r), engine_geometry(g),
                                     torch.from_numpy(data).float(), order=2)
    fo, go_, Ho = go.all_atom_derivs("l2fit", I, x, r, g, data, 2)
    assert abs(loss.item() - fo[0]) <= TOL * abs(fo[0])
    assert entry_relerr(gr_.cpu().numpy(), go_) < TOL
    assert entry_relerr(H.cpu().numpy(), Ho) < TOL


@pytest.mark.parametrize("case", ["2d", "3d"])
def test_l2_single_atom_mode_matches_oracle(eng, cuda_ready, case):
    """Per-atom L2derivs_RadProj(atom, Rad, C): each atom fitted alone to C,
    value includes 1/2 sum C^2 over the whole sinogram."""
    g, I, x, r = _setup(case, seed=5)
    C = go.radproj(I[:1] * 1.1, x[:1], r[:1], g) + 0.01
    C = C.astype(np.float32).astype(np.float64)
    f, gr_, H = eng.atom_derivs(engine_atoms(I, x, r), engine_geometry(g), "l2_atom",
                                torch.from_numpy(C).float(), order=2)
    fo, go_, Ho = [], [], []
    for j in range(I.size):
        a = go.atom_derivs("l2", I[j], x[j], r[j], g, C, 2)
        fo.append(a[0]); go_.append(a[1]); Ho.append(a[2])
    assert relerr(f.cpu().numpy(), np.array(fo)) < TOL
    assert entry_relerr(gr_.cpu().numpy(), np.array(go_)) < TOL
    assert entry_relerr(H.cpu().numpy(), np.array(Ho)) < TOL


@pytest.mark.parametrize("case", ["2d", "3d"])
def test_kl_fit_matches_oracle(eng, cuda_ready, case):
    g, I, x, r = _setup(case, seed=6)
    rng = np.random.default_rng(7)
    b = 0.05
    lam = go.radproj(I, x, r, g) * 200 + b * 200
    counts = rng.poisson(lam).astype(np.float64) / 200
    atoms = engine_atoms(I * 1.05, x, r)
    loss, gr_, H = eng.kl_fit_derivs(atoms, engine_geometry(g),
                                     torch.from_numpy(counts).float(), b, order=2)
    R = go.radproj(I * 1.05, x, r, g)
    assert abs(loss.item() - go.kl_value(counts, R, b)) <= TOL * go.kl_value(counts, R, b)
    al, be = go.kl_fields(counts, R, b)
    fo, go_, Ho = go.all_atom_derivs("field", I * 1.05, x, r, g, al, 2, beta=be)
    assert entry_relerr(gr_.cpu().numpy(), go_) < TOL
    assert entry_relerr(H.cpu().numpy(), Ho) < TOL


def test_bitwise_deterministic(eng, cuda_ready):
    g, I, x, r = _setup("3d", seed=9)
    atoms, geom = engine_atoms(I, x, r), engine_geometry(g)
    data = torch.from_numpy(go.radproj(I, x, r, g) * 0.95).float().cuda()
    outs = []
    for _ in range(2):
        R = eng.radproj(atoms, geom)
        loss, gg, H = eng.l2_fit_derivs(atoms, geom, data, order=2)
        outs.append((R.clone(), loss.clone(), gg.clone(), H.clone()))
    for a, b in zip(*outs):
        assert torch.equal(a, b)


def test_atoms_outside_detector_and_empty(eng, cuda_ready):
    g = make_geometry("2d", 12, 64)
    I, x, r = make_atoms(2, 5, 12)
    x[0] = [5.0, 5.0]    # far outside: projects off the detector
    R = eng.radproj(engine_atoms(I, x, r), engine_geometry(g)).cpu().numpy()
    assert relerr(R, go.radproj(I, x, r, g)) < TOL
    R0 = eng.radproj(engine_atoms(I[:0], x[:0], r[:0]), engine_geometry(g))
    assert torch.count_nonzero(R0).item() == 0


@pytest.mark.parametrize("case", ["2d", "3d"])
@pytest.mark.parametrize("psf", [False, True])
def test_atom_order_does_not_change_results(eng, cuda_ready, case, psf):
    """A processing order (spatial or any permutation) changes only which lane
    visits an atom; outputs stay indexed by atom."""
    g, I, x, r = _setup(case, seed=21)
    geom = engine_geometry(g)
    field = torch.from_numpy(go.radproj(I, x, r, g) * 0.9).float().cuda()
    base = eng.DeviceAtoms(I, x, r)
    f0, g0, H0 = eng.atom_derivs(base, geom, "inner", field, order=2, psf=psf)
    perm = np.random.default_rng(3).permutation(len(I)).astype(np.int32)
    for order in ("spatial", perm):
        atoms = eng.DeviceAtoms(I, x, r, order=order)
        f1, g1, H1 = eng.atom_derivs(atoms, geom, "inner", field, order=2, psf=psf)
        assert entry_relerr(g1.cpu().numpy(), g0.cpu().numpy()) < 1e-6
        assert entry_relerr(H1.cpu().numpy(), H0.cpu().numpy()) < 1e-6
        assert relerr(f1.cpu().numpy(), f0.cpu().numpy()) < 1e-6



@pytest.mark.parametrize("case", ["2d", "3d"])
def test_work_split_does_not_change_results(eng, cuda_ready, case):
    """Every derivative work split (warps, angles per lane group, atoms per
    warp) gives the same per-atom results up to rounding of the chunk sums."""
    import importlib
    tuning = importlib.import_module("2018_dictionary_tomography_gb300.tuning")
    g, I, x, r = _setup(case, seed=23)
    geom, atoms = engine_geometry(g), engine_atoms(I, x, r)
    field = torch.from_numpy(go.radproj(I, x, r, g) * 0.9).float().cuda()
    saved = tuning.get_split()
    saved_lanes = tuning.get_derivative_split()
    saved_one = tuning.get_one_angle_budget()
    try:
        f0, g0, H0 = eng.atom_derivs(atoms, geom, "inner", field, order=2)
        tuning.set_one_angle_budget(0)          # let the target-warps splits take effect
        for split in ((1024, 1, 1), (32768, 2, 2), (4096, 1, 8), (65536, 4, 0)):
            tuning.set_split(*split)
            f1, g1, H1 = eng.atom_derivs(atoms, geom, "inner", field, order=2)
            assert entry_relerr(g1.cpu().numpy(), g0.cpu().numpy()) < 1e-6
            assert entry_relerr(H1.cpu().numpy(), H0.cpu().numpy()) < 1e-6
        tuning.set_split(*saved)
        # cells of a pair walked by 8 (default here), 2 or 1 lanes
        npairs = len(I) * g.shape[0]
        for lanes in (0, 2 * npairs):
            tuning.set_derivative_split(lanes)
            f1, g1, H1 = eng.atom_derivs(atoms, geom, "inner", field, order=2)
            assert relerr(f1.cpu().numpy(), f0.cpu().numpy()) < 1e-6
            assert entry_relerr(g1.cpu().numpy(), g0.cpu().numpy()) < 1e-6
            assert entry_relerr(H1.cpu().numpy(), H0.cpu().numpy()) < 1e-6
    finally:
        tuning.set_split(*saved)
        tuning.set_derivative_split(saved_lanes)
        tuning.set_one_angle_budget(saved_one)


def test_projection_tiling_is_bitwise_neutral(eng, cuda_ready):
    """Both 3D tilings sum every cell over its atoms in index order: the
    sinogram and loss are bitwise equal."""
    import importlib
    tuning = importlib.import_module("2018_dictionary_tomography_gb300.tuning")
    g, I, x, r = _setup("3d", seed=31)
    geom, atoms = engine_geometry(g), engine_atoms(I, x, r)
    data = torch.from_numpy(go.radproj(I, x, r, g) * 1.1).float().cuda()
    outs = []
    try:
        for form in (1, 2):
            tuning.set_projection_tiling(form)
            fw = eng.fit_forward(atoms, geom, data, "l2", want_R=True)
            outs.append((fw["R"].clone(), fw["loss"].clone()))
    finally:
        tuning.set_projection_tiling(1)
    assert torch.equal(outs[0][0], outs[1][0])
    assert relerr(outs[0][0].cpu().numpy(), go.radproj(I, x, r, g)) < TOL


def test_projection_split_over_warps(eng, cuda_ready):
    """Small 3D problems split each tile's atoms over a block's warps; that
    changes only the rounding of the combined cell sums, both tilings still
    agree bitwise, and the projection still matches the oracle."""
    import importlib
    tuning = importlib.import_module("2018_dictionary_tomography_gb300.tuning")
    g = make_geometry("3d", 12, 40, 44)
    I, x, r = make_atoms(3, 300, 33, rdiag=(6.0, 12.0), box=0.7)
    geom, atoms = engine_geometry(g), engine_atoms(I, x, r)
    Ro = go.radproj(I, x, r, g)
    data = torch.from_numpy(Ro * 1.1).float().cuda()
    saved = tuning.get_projection_split()
    outs = {}
    try:
        for split in (1 << 30, 0):
            tuning.set_projection_split(split)
            for form in (1, 2):
                tuning.set_projection_tiling(form)
                fw = eng.fit_forward(atoms, geom, data, "l2", want_R=True)
                outs[(split, form)] = (fw["R"].clone(), float(fw["loss"].item()))
    finally:
        tuning.set_projection_tiling(1)
        tuning.set_projection_split(saved)
    Rs, Ru = outs[(1 << 30, 1)][0], outs[(0, 1)][0]
    assert torch.equal(Rs, outs[(1 << 30, 2)][0])
    assert torch.equal(Ru, outs[(0, 2)][0])
    assert relerr(Rs.cpu().numpy(), Ru.cpu().numpy()) < 1e-6
    assert relerr(Rs.cpu().numpy(), Ro) < TOL
    d32 = (Ro * 1.1).astype(np.float32).astype(np.float64)
    lo = 0.5 * float(np.sum((Ro - d32) ** 2))
    for key, (_R, loss) in outs.items():
        assert abs(loss - lo) <= TOL * lo, key


@pytest.mark.parametrize("case", ["2p5d", "3d"])
def test_wide_row_hessian_walk_matches_oracle(eng, cuda_ready, case):
    """The 3D Hessian kernel's wide-row variant (plan key 8: rows walked in
    8-cell chunks) against the oracle, on atoms whose supports span 5-10
    cells per row, and against the default walk (the cells of a row are
    summed in the same order: equal up to contraction choices)."""
    lib = __import__("importlib").import_module("2018_dictionary_tomography_gb300._lib")
    c = CASES[case]
    g = make_geometry(c["kind"], c["A"], c["D0"], c.get("D1"))
    I, x, r = make_atoms(c["dim"], c["N"], 11, rdiag=(2.0, 4.0), roff=0.5)
    rng = np.random.default_rng(12)
    data = (go.radproj(I * 0.9, x + 0.01, r, g) + rng.normal(0, 0.01, g.shape))
    data = data.astype(np.float32).astype(np.float64)
    atoms, geom = engine_atoms(I, x, r), engine_geometry(g)
    d = torch.from_numpy(data).float().cuda()
    fw = eng.fit_forward(atoms, geom, d, "l2", 0.0)
    plan = eng.Plan(lib.GR_OP_DERIVS_2, atoms, geom).set(8, 1)
    _f, gw, Hw = eng.atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, 2, plan=plan)
    _f, gd, Hd = eng.atom_derivs(atoms, geom, "field", fw["alpha"], None, 1.0, 2)
    _fo, go_, Ho = go.all_atom_derivs("l2fit", I, x, r, g, data, 2)
    assert entry_relerr(gw.cpu().numpy(), go_) < TOL
    assert entry_relerr(Hw.cpu().numpy(), Ho) < TOL
    assert entry_relerr(Hw.cpu().numpy(), Hd.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("form", [2, 3])
def test_2d_two_cells_per_lane_tiles_match_oracle(eng, cuda_ready, form):
    """2D projection with 64- or 128-cell tiles (plan key 3 = 2 or 3: two or
    four cells per lane) against the oracle, on wide and narrow footprints,
    and against the 32-cell tiles (the atoms a cell sums are the same; their
    grouping into passes differs, so the sums agree to FP32 rounding)."""
    lib = __import__("importlib").import_module("2018_dictionary_tomography_gb300._lib")
    g = make_geometry("2d", 40, 300)
    for rdiag in ((0.8, 2.0), (6.0, 12.0)):
        I, x, r = make_atoms(2, 300, 13, rdiag=rdiag, roff=0.3)
        rng = np.random.default_rng(14)
        data = go.radproj(I * 0.9, x, r, g) + rng.normal(0, 0.01, g.shape)
        data = data.astype(np.float32).astype(np.float64)
        atoms, geom = engine_atoms(I, x, r), engine_geometry(g)
        d = torch.from_numpy(data).float().cuda()
        plan = eng.Plan(lib.GR_OP_PROJECT, atoms, geom).set(3, form)
        fw2 = eng.fit_forward(atoms, geom, d, "l2", 0.0, want_R=True, plan=plan)
        fw1 = eng.fit_forward(atoms, geom, d, "l2", 0.0, want_R=True)
        Ro = go.radproj(I, x, r, g)
        assert relerr(fw2["R"].cpu().numpy(), Ro) < TOL
        lo = go.l2_value(Ro, data)
        assert abs(fw2["loss"].item() - lo) <= TOL * abs(lo)
        assert relerr(fw2["R"].cpu().numpy(), fw1["R"].cpu().numpy()) < 1e-6
