"""CPU checks of the C ABI: the library builds, loads and exports every
function include/gauss_radon.h declares.  No compute calls (no GPU here)."""
import ctypes
import importlib
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(gr_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gr_radproj", "gr_fit_forward", "gr_atom_derivs", "gr_workspace_bytes"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load(build_if_missing=True)
    raw = ctypes.CDLL(lib_mod.library_path())
    for name in declared_functions():
        assert hasattr(raw, name), name
    assert lib.gr_version() >= 10000
    assert lib.gr_status_string(-2).decode().startswith("workspace")


def test_workspace_query_and_argument_errors_without_gpu():
    """Host-side validation runs before any device work."""
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load()
    at = lib_mod.GrAtoms()
    at.n_atoms = 0
    g = lib_mod.GrGeometry()
    g.kdet = 3  # invalid
    g.n_angles = 4
    assert lib.gr_workspace_bytes(0, ctypes.byref(at), ctypes.byref(g)) == 0
    rc = lib.gr_radproj(ctypes.byref(at), ctypes.byref(g), None, None, 0, None)
    assert rc == lib_mod.GR_OK - 1  # GR_ERR_ARG


def test_morton_order_is_permutation():
    eng = importlib.import_module("2018_dictionary_tomography_gb300.engine")
    x = np.random.default_rng(0).uniform(-1, 1, (1000, 3))
    p = eng.morton_order(x)
    assert sorted(p.tolist()) == list(range(1000))
    # consecutive atoms along the curve are closer than in index order
    d_curve = np.linalg.norm(np.diff(x[p], axis=0), axis=1).mean()
    d_index = np.linalg.norm(np.diff(x, axis=0), axis=1).mean()
    assert d_curve < 0.5 * d_index


def test_tuning_keys_round_trip_without_gpu():
    """gr_set_tuning / gr_get_tuning: each key keeps a valid value and
    rejects an invalid one (host-side only)."""
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load()
    # key: (a valid value, an invalid value)
    cases = {0: (65536, 16), 1: (2, 0), 2: (4, 3), 3: (3, 4), 4: (1 << 20, -1),
             6: (4096, -5), 7: (0, -1), 8: (1, 2), 9: (1, 2)}
    for key, (good, bad) in cases.items():
        saved = lib.gr_get_tuning(key)
        try:
            assert lib.gr_set_tuning(key, good) == 0, key
            assert lib.gr_get_tuning(key) == good, key
            assert lib.gr_set_tuning(key, bad) == -1, key
            assert lib.gr_get_tuning(key) == good, key
        finally:
            assert lib.gr_set_tuning(key, saved) == 0
    assert lib.gr_get_tuning(99) == -1
    assert lib.gr_set_tuning(99, 1) == -1


def test_fit_loop_calls_reject_bad_arguments_without_gpu():
    """The device-loop calls check their arguments before any CUDA call: a
    null loop is GR_ERR_ARG for every step, including the gated section."""
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load()
    err = lib_mod.GR_OK - 1  # GR_ERR_ARG
    assert lib.gr_fit_loop_gate_begin(None, None, None, None, 1) == err
    assert lib.gr_fit_loop_gate_end(None, None) == err
    assert lib.gr_fit_loop_end(None, None, None, None, None, 1, 1, 1, 0.0, 1, None) == err
    assert lib.gr_fit_loop_instantiate(None) == err
    assert lib.gr_fit_loop_launch(None, None) == err
    assert lib.gr_fit_loop_destroy(None) == lib_mod.GR_OK
    assert lib.gr_fit_loop_begin(None, None, None) == err


def test_plan_create_set_get_without_gpu():
    """gr_plan_*: a caller-owned schedule; argument checks and workspace sizes
    run on the host (sizes only: no pointer is dereferenced)."""
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load()
    at = lib_mod.GrAtoms()
    at.n_atoms = 100
    at.I = at.x = at.r = 16            # non-null stand-ins, never read
    g = lib_mod.GrGeometry()
    g.kdet, g.n_angles, g.frames = 2, 50, 16
    for k in range(2):
        g.n_det[k], g.det[k] = 64, 16
        g.det_first[k], g.det_inv_step[k] = -1.0, 32.0
    h = ctypes.c_void_p()
    assert lib.gr_plan_create(9, ctypes.byref(at), ctypes.byref(g), ctypes.byref(h)) == -1
    assert lib.gr_plan_create(2, ctypes.byref(at), ctypes.byref(g), ctypes.byref(h)) == 0
    assert h.value
    # a copy of the process-wide values, then independent of them
    for key in (0, 1, 2, 3, 4, 6, 7, 8, 9):
        assert lib.gr_plan_get(h, key) == lib.gr_get_tuning(key)
    # the wide-row Hessian walk is a switch (0 or 1)
    assert lib.gr_plan_set(h, 8, 1) == 0 and lib.gr_plan_get(h, 8) == 1
    assert lib.gr_plan_set(h, 8, 2) == -1 and lib.gr_get_tuning(8) == 0
    assert lib.gr_plan_set(h, 8, 0) == 0
    assert lib.gr_plan_set(h, 3, 2) == 0 and lib.gr_plan_get(h, 3) == 2
    assert lib.gr_get_tuning(3) == 1
    assert lib.gr_plan_set(h, 3, 5) == -1 and lib.gr_plan_set(h, 5, 1) == -1
    assert lib.gr_plan_get(h, 5) == -1
    # the workspace follows the plan's schedule (32-row tiles: fewer bitmaps)
    ws_default = lib.gr_workspace_bytes(0, ctypes.byref(at), ctypes.byref(g))
    ws_plan = lib.gr_plan_workspace_bytes(h, 0, ctypes.byref(at), ctypes.byref(g))
    assert 0 < ws_plan < ws_default
    # at least 4 angles per lane group: fewer angle chunks, smaller partials
    assert lib.gr_plan_set(h, 1, 4) == 0 and lib.gr_plan_set(h, 7, 0) == 0
    assert (lib.gr_plan_workspace_bytes(h, 2, ctypes.byref(at), ctypes.byref(g)) <
            lib.gr_workspace_bytes(2, ctypes.byref(at), ctypes.byref(g)))
    assert lib.gr_plan_destroy(h) == 0
    assert lib.gr_radproj_plan(None, ctypes.byref(at), ctypes.byref(g), None, None, 0, None) == -1


def test_skip_forward_items_and_argument_checks_without_gpu():
    """gr_fit_items counts the 3D forward's (angle, tile) items under a plan's
    tiling (0 for 2D); the skipping forward and its record refuse 2D
    geometries and missing data before any device work."""
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load()
    at = lib_mod.GrAtoms()
    at.n_atoms = 100
    at.I = at.x = at.r = 16            # non-null stand-ins, never read
    g = lib_mod.GrGeometry()
    g.kdet, g.n_angles, g.frames = 2, 50, 16
    for k in range(2):
        g.det[k], g.det_first[k], g.det_inv_step[k] = 16, -1.0, 32.0
    g.n_det[0], g.n_det[1] = 70, 65
    n = ctypes.c_size_t()
    assert lib.gr_fit_items(None, ctypes.byref(g), ctypes.byref(n)) == 0
    assert n.value == 50 * 5 * 3                 # 16 x 32 tiles
    h = ctypes.c_void_p()
    assert lib.gr_plan_create(0, ctypes.byref(at), ctypes.byref(g), ctypes.byref(h)) == 0
    assert lib.gr_plan_set(h, 3, 2) == 0
    assert lib.gr_fit_items(h, ctypes.byref(g), ctypes.byref(n)) == 0
    assert n.value == 50 * 3 * 3                 # 32 x 32 tiles
    assert lib.gr_fit_items(h, ctypes.byref(g), None) == -1
    items = n.value
    # no data: refused before any launch
    assert lib.gr_fit_empty_loss(h, ctypes.byref(at), ctypes.byref(g), 1, None, 0.0, 16,
                                 items, None, 0, None) == -1
    assert lib.gr_fit_forward_skip(h, ctypes.byref(at), ctypes.byref(g), 1, None, 0.0, 16,
                                   None, 16, 16, items, None, 0, None) == -1
    # no record: refused
    assert lib.gr_fit_forward_skip(h, ctypes.byref(at), ctypes.byref(g), 1, 16, 0.0, 16,
                                   None, 16, None, items, None, 0, None) == -1
    # a record of another tiling (the default's 750 items against the plan's
    # 450): refused, with data, record and workspace present
    assert lib.gr_fit_empty_loss(h, ctypes.byref(at), ctypes.byref(g), 1, 16, 0.0, 16,
                                 50 * 5 * 3, 16, 1 << 30, None) == -1
    assert lib.gr_fit_forward_skip(h, ctypes.byref(at), ctypes.byref(g), 1, 16, 0.0, 16,
                                   None, 16, 16, 50 * 5 * 3, 16, 1 << 30, None) == -1
    # 2D: no items to skip, and both calls refuse
    g.kdet = 1
    assert lib.gr_fit_items(None, ctypes.byref(g), ctypes.byref(n)) == 0 and n.value == 0
    assert lib.gr_fit_empty_loss(None, ctypes.byref(at), ctypes.byref(g), 1, 16, 0.0, 16,
                                 0, None, 0, None) == -1
    assert lib.gr_fit_forward_skip(None, ctypes.byref(at), ctypes.byref(g), 1, 16, 0.0, 16,
                                   None, 16, 16, 0, None, 0, None) == -1
    assert lib.gr_plan_destroy(h) == 0


def test_batch_layout_without_gpu():
    """gr_batch_workspace_bytes: sizes only (no pointer is dereferenced); a
    member that cannot be batched (3D, or 8 bitmap words and more) gives 0."""
    lib_mod = importlib.import_module("2018_dictionary_tomography_gb300._lib")
    lib = lib_mod.load()

    def member(n, kdet=1, A=30, D=64, iso=1):
        m = lib_mod.GrBatchMember()
        for at in (m.cur, m.trial):
            at.n_atoms, at.I, at.x, at.r, at.r_iso = n, 16, 16, 16, iso
        m.geom.kdet, m.geom.n_angles, m.geom.frames = kdet, A, 16
        for k in range(kdet):
            m.geom.n_det[k], m.geom.det[k] = D, 16
            m.geom.det_first[k], m.geom.det_inv_step[k] = -1.0, D / 2.0
        for name in ("data", "fields", "loss_cur", "loss_trial", "theta", "theta_trial", "lam",
                     "step", "f", "g", "H", "hist", "hist_acc", "counter"):
            setattr(m, name, 16)
        m.hist_len, m.max_iter, m.tol, m.lam_min, m.lam_max = 120, 100, 1e-6, 1e-4, 1e8
        return m

    arr = (lib_mod.GrBatchMember * 3)(member(20), member(100, A=50), member(7, D=300))
    one = lib.gr_batch_workspace_bytes(arr, 1)
    three = lib.gr_batch_workspace_bytes(arr, 3)
    assert one > 0 and three > one and three % 256 == 0
    assert lib.gr_batch_workspace_bytes((lib_mod.GrBatchMember * 1)(member(300)), 1) == 0
    assert lib.gr_batch_workspace_bytes((lib_mod.GrBatchMember * 1)(member(20, kdet=2)), 1) == 0
    bad = member(20)
    bad.counter = None
    assert lib.gr_batch_workspace_bytes((lib_mod.GrBatchMember * 1)(bad), 1) == 0
    h = ctypes.c_void_p()
    assert lib.gr_batch_create(arr, 0, None, 0, 8, None, ctypes.byref(h)) == -1
    assert lib.gr_batch_create(arr, 3, None, 0, 8, None, ctypes.byref(h)) == -1
    assert lib.gr_batch_destroy(None) == 0
