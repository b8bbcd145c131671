"""ctypes binding of the C ABI in include/gauss_radon.h.

The compute path has no fallback: if the CUDA library cannot be built or
loaded, or no CUDA device is present, every engine call raises.
"""
import ctypes
import os
import threading

from . import build_ext

GR_OK = 0
GR_FIT_NONE, GR_FIT_L2, GR_FIT_KL = 0, 1, 2
GR_MODE_FIELD, GR_MODE_L2_ATOM, GR_MODE_INNER = 0, 1, 2
GR_OP_PROJECT, GR_OP_DERIVS_1, GR_OP_DERIVS_2, GR_OP_ATOM_STEP = 0, 1, 2, 3


class GrAtoms(ctypes.Structure):
    _fields_ = [("n_atoms", ctypes.c_int),
                ("I", ctypes.c_void_p),
                ("x", ctypes.c_void_p),
                ("r", ctypes.c_void_p),
                ("r_iso", ctypes.c_int),
                ("order", ctypes.c_void_p)]


class GrGeometry(ctypes.Structure):
    _fields_ = [("kdet", ctypes.c_int),
                ("n_angles", ctypes.c_int),
                ("frames", ctypes.c_void_p),
                ("n_det", ctypes.c_int * 2),
                ("det", ctypes.c_void_p * 2),
                ("det_first", ctypes.c_float * 2),
                ("det_inv_step", ctypes.c_float * 2)]


class GrBatchMember(ctypes.Structure):
    """gr_batch_member: one 2D fit of a batch (device pointers)."""
    _fields_ = [("cur", GrAtoms),
                ("trial", GrAtoms),
                ("geom", GrGeometry),
                ("data", ctypes.c_void_p),
                ("fields", ctypes.c_void_p),
                ("loss_cur", ctypes.c_void_p),
                ("loss_trial", ctypes.c_void_p),
                ("theta", ctypes.c_void_p),
                ("theta_trial", ctypes.c_void_p),
                ("lam", ctypes.c_void_p),
                ("step", ctypes.c_void_p),
                ("f", ctypes.c_void_p),
                ("g", ctypes.c_void_p),
                ("H", ctypes.c_void_p),
                ("hist", ctypes.c_void_p),
                ("hist_acc", ctypes.c_void_p),
                ("counter", ctypes.c_void_p),
                ("hist_len", ctypes.c_int),
                ("max_iter", ctypes.c_int),
                ("tol", ctypes.c_double),
                ("lam_min", ctypes.c_double),
                ("lam_max", ctypes.c_double)]


class EngineError(RuntimeError):
    pass


EXPORTS = ("gr_version", "gr_preload", "gr_status_string", "gr_workspace_bytes", "gr_radproj",
           "gr_fit_forward", "gr_atom_derivs", "gr_count_support", "gr_probe_ex2",
           "gr_launch_count", "gr_atom_step", "gr_newton_solve", "gr_volproj", "gr_newton_accept",
           "gr_psf_radproj", "gr_psf_fit_forward", "gr_psf_atom_derivs", "gr_psf_volproj",
           "gr_set_tuning", "gr_get_tuning", "gr_kernel_timer", "gr_kernel_timer_read",
           "gr_fit_loop_begin", "gr_fit_loop_end", "gr_fit_loop_gate_begin",
           "gr_fit_loop_gate_end", "gr_fit_loop_instantiate",
           "gr_fit_loop_launch", "gr_fit_loop_destroy", "gr_regulariser",
           "gr_sino_moments", "gr_accept_fields", "gr_newton_accept_fields",
           "gr_plan_create", "gr_plan_destroy", "gr_plan_set", "gr_plan_get",
           "gr_plan_workspace_bytes", "gr_radproj_plan", "gr_fit_forward_plan",
           "gr_atom_derivs_plan", "gr_batch_workspace_bytes", "gr_batch_create",
           "gr_batch_prologue", "gr_batch_iterate", "gr_fit_loop_end_open", "gr_batch_destroy",
           "gr_fit_items", "gr_fit_empty_loss", "gr_fit_forward_skip")

_lock = threading.Lock()
_lib = None


def library_path():
    return build_ext.LIB


def load(build_if_missing=True):
    """Load libgauss_radon.so (building it first when allowed)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = build_ext.LIB
        if build_if_missing:
            path = build_ext.build()
        if not os.path.exists(path):
            raise EngineError("CUDA engine library not built: %s" % path)
        lib = ctypes.CDLL(path)
        P = ctypes.POINTER
        lib.gr_version.restype = ctypes.c_int
        lib.gr_preload.restype = ctypes.c_int
        lib.gr_preload.argtypes = []
        lib.gr_status_string.restype = ctypes.c_char_p
        lib.gr_status_string.argtypes = [ctypes.c_int]
        lib.gr_workspace_bytes.restype = ctypes.c_size_t
        lib.gr_workspace_bytes.argtypes = [ctypes.c_int, P(GrAtoms), P(GrGeometry)]
        lib.gr_radproj.restype = ctypes.c_int
        lib.gr_radproj.argtypes = [P(GrAtoms), P(GrGeometry), ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.gr_fit_forward.restype = ctypes.c_int
        lib.gr_fit_forward.argtypes = [P(GrAtoms), P(GrGeometry), ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_float,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_void_p]
        lib.gr_atom_derivs.restype = ctypes.c_int
        lib.gr_atom_derivs.argtypes = [P(GrAtoms), P(GrGeometry), ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_float, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_size_t, ctypes.c_void_p]
        lib.gr_count_support.restype = ctypes.c_int
        lib.gr_count_support.argtypes = [P(GrAtoms), P(GrGeometry), ctypes.c_void_p,
                                         ctypes.c_void_p]
        lib.gr_probe_ex2.restype = ctypes.c_int
        lib.gr_probe_ex2.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_void_p]
        lib.gr_atom_step.restype = ctypes.c_int
        lib.gr_atom_step.argtypes = [P(GrAtoms), P(GrAtoms), P(GrGeometry), ctypes.c_int,
                                     ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                     ctypes.c_void_p]
        lib.gr_newton_solve.restype = ctypes.c_int
        lib.gr_newton_solve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + \
            [ctypes.c_void_p] * 12
        lib.gr_newton_accept.restype = ctypes.c_int
        lib.gr_newton_accept.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_void_p] * 5 +
                                         [ctypes.c_double] * 2 + [ctypes.c_void_p] * 9 +
                                         [ctypes.c_int, ctypes.c_void_p])
        lib.gr_newton_accept_fields.restype = ctypes.c_int
        lib.gr_newton_accept_fields.argtypes = (
            [ctypes.c_int] * 3 + [ctypes.c_void_p] * 5 + [ctypes.c_double] * 2 +
            [ctypes.c_void_p] * 9 + [ctypes.c_int] + [ctypes.c_void_p] * 4 +
            [ctypes.c_size_t, ctypes.c_void_p])
        lib.gr_volproj.restype = ctypes.c_int
        lib.gr_volproj.argtypes = [P(GrAtoms), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p]
        lib.gr_psf_radproj.restype = ctypes.c_int
        lib.gr_psf_radproj.argtypes = lib.gr_radproj.argtypes
        lib.gr_psf_fit_forward.restype = ctypes.c_int
        lib.gr_psf_fit_forward.argtypes = lib.gr_fit_forward.argtypes
        lib.gr_psf_atom_derivs.restype = ctypes.c_int
        lib.gr_psf_atom_derivs.argtypes = lib.gr_atom_derivs.argtypes
        lib.gr_psf_volproj.restype = ctypes.c_int
        lib.gr_psf_volproj.argtypes = [P(GrAtoms), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
        lib.gr_set_tuning.restype = ctypes.c_int
        lib.gr_set_tuning.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.gr_get_tuning.restype = ctypes.c_int
        lib.gr_get_tuning.argtypes = [ctypes.c_int]
        lib.gr_kernel_timer.restype = ctypes.c_int
        lib.gr_kernel_timer.argtypes = [ctypes.c_int, ctypes.c_int]
        vp = ctypes.c_void_p
        lib.gr_accept_fields.restype = ctypes.c_int
        lib.gr_accept_fields.argtypes = [vp, vp, vp, vp, vp, vp, ctypes.c_size_t, vp]
        lib.gr_sino_moments.restype = ctypes.c_int
        lib.gr_sino_moments.argtypes = [ctypes.POINTER(GrGeometry), vp, vp, ctypes.c_float,
                                        ctypes.c_float, vp, vp, vp, vp]
        lib.gr_regulariser.restype = ctypes.c_int
        lib.gr_regulariser.argtypes = [ctypes.c_int, vp, ctypes.c_int, ctypes.POINTER(GrAtoms),
                                       ctypes.c_int, vp, vp, vp, ctypes.c_int, vp]
        lib.gr_fit_loop_begin.restype = ctypes.c_int
        lib.gr_fit_loop_begin.argtypes = [vp, vp, ctypes.POINTER(vp)]
        lib.gr_fit_loop_end.restype = ctypes.c_int
        lib.gr_fit_loop_end.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_int, vp]
        lib.gr_fit_loop_gate_begin.restype = ctypes.c_int
        lib.gr_fit_loop_gate_begin.argtypes = [vp, vp, vp, vp, ctypes.c_int]
        lib.gr_fit_loop_gate_end.restype = ctypes.c_int
        lib.gr_fit_loop_gate_end.argtypes = [vp, vp]
        lib.gr_fit_loop_instantiate.restype = ctypes.c_int
        lib.gr_fit_loop_instantiate.argtypes = [vp]
        lib.gr_fit_loop_launch.restype = ctypes.c_int
        lib.gr_fit_loop_launch.argtypes = [vp, vp]
        lib.gr_fit_loop_destroy.restype = ctypes.c_int
        lib.gr_fit_loop_destroy.argtypes = [vp]
        bm = ctypes.POINTER(GrBatchMember)
        lib.gr_batch_workspace_bytes.restype = ctypes.c_size_t
        lib.gr_batch_workspace_bytes.argtypes = [bm, ctypes.c_int]
        lib.gr_batch_create.restype = ctypes.c_int
        lib.gr_batch_create.argtypes = [bm, ctypes.c_int, vp, ctypes.c_size_t, ctypes.c_int, vp,
                                        ctypes.POINTER(vp)]
        lib.gr_batch_prologue.restype = ctypes.c_int
        lib.gr_batch_prologue.argtypes = [vp, vp]
        lib.gr_batch_iterate.restype = ctypes.c_int
        lib.gr_batch_iterate.argtypes = [vp, vp, vp]
        lib.gr_fit_loop_end_open.restype = ctypes.c_int
        lib.gr_fit_loop_end_open.argtypes = [vp, vp]
        lib.gr_batch_destroy.restype = ctypes.c_int
        lib.gr_batch_destroy.argtypes = [vp]
        lib.gr_kernel_timer_read.restype = ctypes.c_int
        lib.gr_kernel_timer_read.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_int)]
        lib.gr_launch_count.restype = ctypes.c_ulonglong
        lib.gr_launch_count.argtypes = []
        lib.gr_plan_create.restype = ctypes.c_int
        lib.gr_plan_create.argtypes = [ctypes.c_int, P(GrAtoms), P(GrGeometry), ctypes.POINTER(vp)]
        lib.gr_plan_destroy.restype = ctypes.c_int
        lib.gr_plan_destroy.argtypes = [vp]
        lib.gr_plan_set.restype = ctypes.c_int
        lib.gr_plan_set.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        lib.gr_plan_get.restype = ctypes.c_int
        lib.gr_plan_get.argtypes = [vp, ctypes.c_int]
        lib.gr_plan_workspace_bytes.restype = ctypes.c_size_t
        lib.gr_plan_workspace_bytes.argtypes = [vp, ctypes.c_int, P(GrAtoms), P(GrGeometry)]
        lib.gr_radproj_plan.restype = ctypes.c_int
        lib.gr_radproj_plan.argtypes = [vp] + lib.gr_radproj.argtypes
        lib.gr_fit_forward_plan.restype = ctypes.c_int
        lib.gr_fit_forward_plan.argtypes = [vp] + lib.gr_fit_forward.argtypes
        lib.gr_atom_derivs_plan.restype = ctypes.c_int
        lib.gr_atom_derivs_plan.argtypes = [vp] + lib.gr_atom_derivs.argtypes
        lib.gr_fit_items.restype = ctypes.c_int
        lib.gr_fit_items.argtypes = [vp, P(GrGeometry), P(ctypes.c_size_t)]
        lib.gr_fit_empty_loss.restype = ctypes.c_int
        lib.gr_fit_empty_loss.argtypes = [vp, P(GrAtoms), P(GrGeometry), ctypes.c_int, vp,
                                          ctypes.c_float, vp, ctypes.c_size_t, vp,
                                          ctypes.c_size_t, vp]
        lib.gr_fit_forward_skip.restype = ctypes.c_int
        lib.gr_fit_forward_skip.argtypes = [vp, P(GrAtoms), P(GrGeometry), ctypes.c_int, vp,
                                            ctypes.c_float, vp, vp, vp, vp, ctypes.c_size_t,
                                            vp, ctypes.c_size_t, vp]
        _lib = lib
        return lib


def check(status, what):
    if status != GR_OK:
        msg = load().gr_status_string(int(status)).decode()
        raise EngineError("%s failed: %s (status %d)" % (what, msg, status))
