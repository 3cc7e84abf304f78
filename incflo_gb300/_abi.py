"""ctypes binding of the C ABI in include/incflo_gb300.h (the Python-side stub a caller binds).

Loads the in-tree libincflo_gb300.so. There is no fallback: if the library or a CUDA device is
missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libincflo_gb300.so")

GBP_OK, GBP_NOT_CONVERGED, GBP_NAN, GBP_BAD_ARG, GBP_CUDA_ERROR, GBP_TIMEOUT, GBP_NO_DEVICE = range(7)
GBP_NODAL, GBP_MAC = 0, 1
BC_PERIODIC, BC_DIRICHLET, BC_NEUMANN, BC_INFLOW, BC_ROBIN = range(5)
PREC_FP64, PREC_MIXED = 0, 1

# every symbol include/incflo_gb300.h declares
EXPORTS = (
    "gbp_abi_version", "gbp_status_string", "gbp_last_error", "gbp_device_check",
    "gbp_options_default", "gbp_options_set", "gbp_options_parse",
    "gbp_plan_create", "gbp_plan_destroy", "gbp_plan_set_options", "gbp_plan_device_bytes",
    "gbp_nodal_set_sigma_from_density", "gbp_nodal_set_sigma", "gbp_nodal_project",
    "gbp_apply_nodal_projection", "gbp_mac_set_beta", "gbp_mac_set_beta_from_density",
    "gbp_mac_project", "gbp_mac_get_fluxes", "gbp_apply_nodal_projection_host", "gbp_plan_time_kernel", "gbp_plan_check_level_kernels", "gbp_plan_check_coarse_cycle",
    "gbp_nodal_divergence", "gbp_nodal_divergence_noalloc", "gbp_nodal_set_overset_mask",
    "gbp_mac_set_robin", "gbp_mac_set_eb", "gbp_average_down",
    "gbp_amr_create", "gbp_amr_destroy", "gbp_amr_set_options", "gbp_amr_device_bytes",
    "gbp_amr_apply_nodal_projection", "gbp_abec_set_coeffs", "gbp_abec_solve", "gbp_abec_set_coeffs_eta", "gbp_nodal_set_eb", "gbp_nodal_set_eb_inflow", "gbp_mac_set_eb_inflow",
    "gbp_apply_nodal_projection_boxes", "gbp_mac_set_beta_from_density_boxes", "gbp_mac_project_boxes", "gbp_apply_cc_projection", "gbp_enforce_inout_solvability", "gbp_mac_enforce_inout_solvability",
    "gbp_tensor_create", "gbp_tensor_destroy", "gbp_tensor_set_options", "gbp_tensor_device_bytes",
    "gbp_tensor_set_coeffs", "gbp_tensor_solve", "gbp_tensor_apply",
    "gbp_nn_conv3d", "gbp_nn_conv3d_wgrad",
    "gbp_surrogate_create", "gbp_surrogate_destroy", "gbp_surrogate_num_params", "gbp_surrogate_get_params",
    "gbp_surrogate_set_params", "gbp_surrogate_get_grads", "gbp_surrogate_save", "gbp_surrogate_load",
    "gbp_surrogate_train_pair", "gbp_surrogate_predict", "gbp_surrogate_add_sample", "gbp_surrogate_train_step", "gbp_surrogate_num_samples",
    "gbp_surrogate_clear_samples", "gbp_surrogate_train", "gbp_plan_set_surrogate",
)


class Array4(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("lo", ctypes.c_int * 3),
        ("hi", ctypes.c_int * 3),
        ("ncomp", ctypes.c_int),
        ("jstride", ctypes.c_longlong),
        ("kstride", ctypes.c_longlong),
        ("nstride", ctypes.c_longlong),
    ]


class IArray4(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("lo", ctypes.c_int * 3),
        ("hi", ctypes.c_int * 3),
        ("jstride", ctypes.c_longlong),
        ("kstride", ctypes.c_longlong),
    ]


class Geometry(ctypes.Structure):
    _fields_ = [
        ("n_cell", ctypes.c_int * 3),
        ("prob_lo", ctypes.c_double * 3),
        ("prob_hi", ctypes.c_double * 3),
    ]


class Options(ctypes.Structure):
    _fields_ = [
        ("rtol", ctypes.c_double),
        ("atol", ctypes.c_double),
        ("max_coarsening_level", ctypes.c_int),
        ("maxiter", ctypes.c_int),
        ("bottom_maxiter", ctypes.c_int),
        ("bottom_rtol", ctypes.c_double),
        ("bottom_atol", ctypes.c_double),
        ("verbose", ctypes.c_int),
        ("bottom_verbose", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("nu1", ctypes.c_int),
        ("nu2", ctypes.c_int),
        ("omega", ctypes.c_double),
        ("ir_inner_cycles", ctypes.c_int),
        ("use_graphs", ctypes.c_int),
        ("always_use_bnorm", ctypes.c_int),
        ("initial_guess", ctypes.c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("vcycles", ctypes.c_int),
        ("outer_iters", ctypes.c_int),
        ("num_levels", ctypes.c_int),
        ("rhs_norm", ctypes.c_double),
        ("initial_rel_resid", ctypes.c_double),
        ("final_rel_resid", ctypes.c_double),
        ("ms_total", ctypes.c_double),
        ("ms_solve", ctypes.c_double),
        ("kernel_launches", ctypes.c_longlong),
        ("warm_start", ctypes.c_int),
        ("warm_rel_resid", ctypes.c_double),
        ("ms_warm", ctypes.c_double),
        ("prev_rel_resid", ctypes.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None


def load(path: str = LIB_PATH):
    """Load the shared library and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with incflo_gb300.build.build()")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    A4 = ctypes.POINTER(Array4)
    i, d = ctypes.c_int, ctypes.c_double
    sig = {
        "gbp_abi_version": (i, []),
        "gbp_status_string": (ctypes.c_char_p, [i]),
        "gbp_last_error": (ctypes.c_char_p, []),
        "gbp_device_check": (i, []),
        "gbp_options_default": (i, [i, ctypes.POINTER(Options)]),
        "gbp_options_set": (i, [ctypes.POINTER(Options), ctypes.c_char_p, ctypes.c_char_p]),
        "gbp_options_parse": (i, [ctypes.POINTER(Options), ctypes.c_char_p, ctypes.c_char_p]),
        "gbp_plan_create": (i, [ctypes.POINTER(Geometry), i, ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(Options), P,
                                ctypes.POINTER(P)]),
        "gbp_plan_destroy": (i, [P]),
        "gbp_plan_set_options": (i, [P, ctypes.POINTER(Options)]),
        "gbp_plan_device_bytes": (ctypes.c_size_t, [P]),
        "gbp_nodal_set_sigma_from_density": (i, [P, A4, d, d]),
        "gbp_nodal_set_sigma": (i, [P, A4, d]),
        "gbp_nodal_project": (i, [P, A4, A4, A4, i, ctypes.POINTER(Stats)]),
        "gbp_apply_nodal_projection": (i, [P, A4, A4, A4, d, A4, A4, d, d, d, d, i, i,
                                           ctypes.POINTER(Stats)]),
        "gbp_mac_set_beta": (i, [P, A4, A4, A4, d]),
        "gbp_mac_set_beta_from_density": (i, [P, A4, d]),
        "gbp_mac_project": (i, [P, A4, A4, A4, A4, i, ctypes.POINTER(Stats)]),
        "gbp_mac_get_fluxes": (i, [P, A4, A4, A4, A4]),
        "gbp_apply_nodal_projection_host": (i, [P, P, P, d, P, P, d, i, ctypes.POINTER(Stats)]),
        "gbp_plan_time_kernel": (i, [P, i, i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
        "gbp_plan_check_level_kernels": (i, [P, ctypes.POINTER(ctypes.c_double)]),
        "gbp_plan_check_coarse_cycle": (i, [P, ctypes.POINTER(ctypes.c_double)]),
        "gbp_nodal_divergence": (i, [P, A4, i, A4, ctypes.POINTER(ctypes.c_double)]),
        "gbp_nodal_divergence_noalloc": (i, [ctypes.POINTER(Geometry), ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int), A4, i, A4,
                                             ctypes.POINTER(ctypes.c_double), P]),
        "gbp_mac_set_robin": (i, [P, A4, A4, A4]),
        "gbp_mac_set_eb": (i, [P, A4, A4, A4, A4, A4, A4, A4]),
        "gbp_amr_create": (i, [ctypes.POINTER(Geometry), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int), i, ctypes.POINTER(Options), P, ctypes.POINTER(P)]),
        "gbp_amr_destroy": (i, [P]),
        "gbp_abec_set_coeffs": (i, [P, d, A4, d, d, A4, A4, A4, d]),
        "gbp_abec_solve": (i, [P, A4, A4, ctypes.POINTER(Stats)]),
        "gbp_abec_set_coeffs_eta": (i, [P, d, A4, d, d, A4]),
        "gbp_nodal_set_eb": (i, [P, A4]),
        "gbp_nodal_set_eb_inflow": (i, [P, A4, A4, A4]),
        "gbp_mac_set_eb_inflow": (i, [P, A4]),
        "gbp_apply_nodal_projection_boxes": (i, [P, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(A4),
                                                 ctypes.POINTER(A4), ctypes.POINTER(A4), d, ctypes.POINTER(A4),
                                                 ctypes.POINTER(A4), d, d, d, d, i, i, ctypes.POINTER(Stats)]),
        "gbp_mac_set_beta_from_density_boxes": (i, [P, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(A4), d]),
        "gbp_mac_project_boxes": (i, [P, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(A4), ctypes.POINTER(A4),
                                      ctypes.POINTER(A4), ctypes.POINTER(A4), i, ctypes.POINTER(Stats)]),
        "gbp_amr_set_options": (i, [P, ctypes.POINTER(Options)]),
        "gbp_amr_device_bytes": (ctypes.c_size_t, [P]),
        "gbp_amr_apply_nodal_projection": (i, [P, A4, A4, A4, A4, A4, ctypes.POINTER(A4), ctypes.POINTER(A4),
                                               ctypes.POINTER(A4), ctypes.POINTER(A4), ctypes.POINTER(A4), d, d, i,
                                               ctypes.POINTER(Stats)]),
        "gbp_nodal_set_overset_mask": (i, [P, ctypes.POINTER(IArray4)]),
        "gbp_tensor_create": (i, [ctypes.POINTER(Geometry), ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(Options), P, ctypes.POINTER(P)]),
        "gbp_tensor_destroy": (i, [P]),
        "gbp_tensor_set_options": (i, [P, ctypes.POINTER(Options)]),
        "gbp_tensor_device_bytes": (ctypes.c_size_t, [P]),
        "gbp_tensor_set_coeffs": (i, [P, d, A4, d, d, A4, A4, A4, A4, d]),
        "gbp_tensor_solve": (i, [P, A4, A4, ctypes.POINTER(Stats)]),
        "gbp_tensor_apply": (i, [P, A4, A4]),
        "gbp_average_down": (i, [A4, A4, ctypes.POINTER(ctypes.c_int), i, ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_int), P]),
        "gbp_apply_cc_projection": (i, [P, A4, A4, A4, d, A4, A4, A4, A4, A4, d, d, d, d, i, i,
                                        ctypes.POINTER(Stats)]),
        "gbp_enforce_inout_solvability": (i, [P, A4, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_double)]),
        "gbp_mac_enforce_inout_solvability": (i, [P, A4, A4, A4, ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
        "gbp_nn_conv3d": (i, [ctypes.POINTER(ctypes.c_int), i, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_int), P,
                              i, i, i, P, i, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(ctypes.c_int),
                              i, P]),
        "gbp_nn_conv3d_wgrad": (i, [ctypes.POINTER(ctypes.c_int), P, i, i, i, P, i, i, P, P]),
        "gbp_surrogate_create": (i, [i, ctypes.c_ulonglong, ctypes.POINTER(P)]),
        "gbp_surrogate_destroy": (i, [P]),
        "gbp_surrogate_num_params": (ctypes.c_longlong, [P]),
        "gbp_surrogate_get_params": (i, [P, P, ctypes.c_longlong]),
        "gbp_surrogate_set_params": (i, [P, P, ctypes.c_longlong]),
        "gbp_surrogate_get_grads": (i, [P, P, ctypes.c_longlong]),
        "gbp_surrogate_save": (i, [P, ctypes.c_char_p]),
        "gbp_surrogate_load": (i, [P, ctypes.c_char_p]),
        "gbp_surrogate_train_pair": (i, [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), P, P,
                                         ctypes.c_float, ctypes.POINTER(ctypes.c_double), P]),
        "gbp_surrogate_predict": (i, [P, ctypes.POINTER(ctypes.c_int), P, P, P]),
        "gbp_surrogate_add_sample": (i, [P, P, A4]),
        "gbp_surrogate_train_step": (i, [P, P, A4, ctypes.c_float, ctypes.POINTER(ctypes.c_double)]),
        "gbp_surrogate_num_samples": (i, [P]),
        "gbp_surrogate_clear_samples": (i, [P]),
        "gbp_surrogate_train": (i, [P, i, ctypes.c_float, ctypes.c_ulonglong, P, P]),
        "gbp_plan_set_surrogate": (i, [P, P, i, i]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class ProjectionError(RuntimeError):
    def __init__(self, status: int, where: str):
        L = load()
        msg = L.gbp_last_error().decode(errors="replace")
        super().__init__(f"{where}: {L.gbp_status_string(status).decode()} ({status}): {msg}")
        self.status = status


def check(status: int, where: str, allow_not_converged: bool = False) -> int:
    if status == GBP_OK or (allow_not_converged and status == GBP_NOT_CONVERGED):
        return status
    raise ProjectionError(status, where)


def default_options(kind: int) -> Options:
    o = Options()
    check(load().gbp_options_default(kind, ctypes.byref(o)), "gbp_options_default")
    return o
