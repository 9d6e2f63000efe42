"""ctypes binding of the native library ``librsg.so`` (the C ABI declared in include/rsg.h).

There is no CPU fallback: if the library is missing it is built from ressim_gb300/csrc (nvcc required); if that
fails the import error is raised to the caller.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

RSG_OK, RSG_EINVAL, RSG_ECUDA, RSG_ENOMEM, RSG_ESTATE, RSG_ETIMEOUT, RSG_EBREAKDOWN, RSG_ENOTCONV = 0, -1, -2, -3, -4, -5, -6, 1
PREC = {"bilu0": 0, "cpr": 1, "jacobi": 2, "cpr_device": 3, "mcbilu0": 4}
KRYLOV = {"bicgstab": 0, "gmres": 1}
PRECISION = {"fp64": 0, "mixed": 1, "mixed_f32": 2}
SWEEP = {"auto": 0, "cta": 1, "grid": 2, "split": 3}

# every symbol include/rsg.h declares
EXPORTS = [
    "rsg_default_options", "rsg_last_error", "rsg_version", "rsg_create", "rsg_destroy", "rsg_set_matrix", "rsg_set_batch",
    "rsg_setup", "rsg_solve", "rsg_solve_device", "rsg_solve_refined", "rsg_batch_results", "rsg_batch_status", "rsg_amg_level_sizes", "rsg_spmv", "rsg_spmv_device", "rsg_precond_apply",
    "rsg_precond_apply_device", "rsg_get_factors", "rsg_get_stats", "rsg_stream", "rsg_wellschur_reduce", "rsg_wellschur_recover",
    "rsg_spmv_level_probe", "rsg_precond_level_probe", "rsg_spmv_dot_noalloc", "rsg_release", "rsg_server_create",
    "rsg_server_destroy", "rsg_submit", "rsg_submit_view", "rsg_poll", "rsg_server_load", "rsg_request_bytes", "rsg_tuning",
    "rsg_set_jacobian", "rsg_set_jacobian_batch", "rsg_set_jacobian_device", "rsg_solve_jacobian", "rsg_solve_jacobian_device",
    "rsg_get_matrix", "rsg_matrix_size", "rsg_server_hold", "rsg_bo_create", "rsg_bo_assemble", "rsg_bo_assemble_host", "rsg_bo_destroy",
]


class Options(C.Structure):
    _fields_ = [("precond", C.c_int), ("krylov", C.c_int), ("restart", C.c_int), ("precision", C.c_int),
                ("gmres_fallback", C.c_int), ("check_every", C.c_int), ("use_graphs", C.c_int), ("device", C.c_int),
                ("mem_budget", C.c_size_t), ("sweep", C.c_int), ("fma", C.c_int), ("sweep_inflight", C.c_int),
                ("autotune", C.c_int), ("vcycle_form", C.c_int), ("cpr2_threads", C.c_int)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("rel_residual", C.c_double), ("true_rel_residual", C.c_double),
                ("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double), ("device_bytes", C.c_size_t),
                ("start_ms", C.c_double), ("end_ms", C.c_double), ("slot", C.c_int), ("precond", C.c_int), ("batch", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("rel_residual", C.c_double), ("true_rel_residual", C.c_double),
                ("setup_ms", C.c_double), ("solve_ms", C.c_double), ("regularised_blocks", C.c_int), ("amg_levels", C.c_int),
                ("device_bytes", C.c_size_t), ("kernel_launches", C.c_longlong), ("escalated_systems", C.c_int)]


class Table(C.Structure):
    _fields_ = [("n", C.c_int), ("x", C.c_void_p), ("y", C.c_void_p), ("clamp", C.c_int)]


class BoGrid(C.Structure):
    _fields_ = [("na", C.c_int), ("nv", C.c_int), ("nconn", C.c_int), ("adj_start", C.c_void_p), ("adj_nbr", C.c_void_p),
                ("adj_conn", C.c_void_p), ("conn_a", C.c_void_p), ("conn_trans", C.c_void_p), ("conn_ddepth", C.c_void_p),
                ("pore_vol", C.c_void_p), ("gravity", C.c_double), ("i_sw", C.c_int), ("i_x", C.c_int), ("eq", C.c_int * 3)]


class BoFluid(C.Structure):
    _fields_ = [("water", C.c_int), ("oil", C.c_int), ("gas", C.c_int), ("live", C.c_int), ("vap", C.c_int),
                ("pvtw", C.c_double * 5), ("rock", C.c_double * 2), ("rho_sc", C.c_double * 3), ("gas_factor", C.c_double),
                ("rs_of_p", Table), ("pb_of_rs", Table), ("dead_b", Table), ("dead_bmu", Table), ("gas_b", Table),
                ("gas_bmu", Table), ("nsat", C.c_int), ("sat_rs", C.c_void_p), ("sat_b", C.c_void_p), ("sat_bmu", C.c_void_p),
                ("under_b", C.c_void_p), ("under_bmu", C.c_void_p)]


class BoSatfun(C.Structure):
    _fields_ = [("krw", Table), ("krow", Table), ("pcow", Table), ("krg", Table), ("krog", Table), ("pcog", Table),
                ("swco", C.c_double), ("kro_model", C.c_int), ("water", C.c_int), ("gas", C.c_int), ("three_point", C.c_int)]


class RsgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"rsg error {code}: {msg}")
        self.code = code


_LIB = None


def load(build_if_missing: bool = True):
    """Load (building if needed) ``librsg.so``."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError("librsg.so is not built (run __graft_entry__.build())")
        _build.build()
    L = C.CDLL(path)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.rsg_default_options.argtypes = [C.POINTER(Options)]
    L.rsg_last_error.restype = C.c_char_p
    L.rsg_version.restype = C.c_char_p
    L.rsg_create.argtypes = [C.POINTER(vp), C.POINTER(Options)]
    L.rsg_destroy.argtypes = [vp]
    L.rsg_set_matrix.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp]
    L.rsg_set_batch.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp]
    L.rsg_setup.argtypes = [vp, vp]
    L.rsg_solve.argtypes = [vp, vp, vp, C.c_double, C.c_int, ip, dp]
    L.rsg_solve_device.argtypes = [vp, vp, vp, C.c_double, C.c_int, ip, dp]
    L.rsg_solve_refined.argtypes = [vp, vp, vp, C.c_double, C.c_int, C.c_int, ip, dp]
    L.rsg_batch_results.argtypes = [vp, vp, vp, vp]
    L.rsg_batch_status.argtypes = [vp, vp]
    L.rsg_amg_level_sizes.argtypes = [vp, C.c_int, vp, vp, vp]
    L.rsg_spmv.argtypes = [vp, vp, vp]
    L.rsg_spmv_device.argtypes = [vp, vp, vp]
    L.rsg_precond_apply.argtypes = [vp, vp, vp]
    L.rsg_precond_apply_device.argtypes = [vp, vp, vp]
    L.rsg_spmv_dot_noalloc.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    L.rsg_spmv_level_probe.argtypes = [vp, C.c_int]
    L.rsg_precond_level_probe.argtypes = [vp, C.c_int]
    L.rsg_get_factors.argtypes = [vp, vp]
    L.rsg_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.rsg_stream.argtypes = [vp]
    L.rsg_stream.restype = vp
    L.rsg_wellschur_reduce.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, ip, vp, vp, vp, vp]
    L.rsg_wellschur_recover.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
    L.rsg_release.argtypes = [vp]
    L.rsg_server_create.argtypes = [C.POINTER(vp), C.POINTER(Options), C.c_int, C.c_size_t]
    L.rsg_server_destroy.argtypes = [vp]
    L.rsg_submit.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, C.c_double, C.c_int]
    L.rsg_submit_view.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, C.c_double, C.c_int]
    L.rsg_poll.argtypes = [vp, C.c_longlong, C.c_int, vp, C.POINTER(Result)]
    L.rsg_server_load.argtypes = [vp, ip, ip, C.POINTER(C.c_size_t)]
    L.rsg_request_bytes.argtypes = [C.POINTER(Options), C.c_int, C.c_longlong]
    L.rsg_tuning.argtypes = [vp, C.c_char_p, C.c_int]
    L.rsg_set_jacobian.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int]
    L.rsg_set_jacobian_batch.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
    L.rsg_set_jacobian_device.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int]
    L.rsg_solve_jacobian.argtypes = [vp, vp, vp, C.c_double, C.c_int, ip, dp]
    L.rsg_solve_jacobian_device.argtypes = [vp, vp, vp, C.c_double, C.c_int, ip, dp]
    L.rsg_get_matrix.argtypes = [vp, vp, vp, vp]
    L.rsg_server_hold.argtypes = [vp, C.c_int]
    L.rsg_matrix_size.argtypes = [vp, ip, C.POINTER(C.c_longlong)]
    L.rsg_bo_create.argtypes = [C.POINTER(vp), C.POINTER(BoGrid), C.POINTER(BoFluid), C.POINTER(BoSatfun), C.c_int, C.c_int, vp, vp,
                                C.c_int]
    L.rsg_bo_assemble.argtypes = [vp, vp, vp, vp, vp, vp, C.c_double, C.c_int, vp, vp, C.c_int, vp, vp, vp, vp, vp]
    L.rsg_bo_assemble_host.argtypes = [vp, vp, vp, vp, vp, vp, C.c_double, C.c_int, vp, vp, C.c_int, vp, vp, vp, vp]
    L.rsg_bo_destroy.argtypes = [vp]
    for name in EXPORTS:
        getattr(L, name).restype = getattr(L, name).restype if name in ("rsg_last_error", "rsg_version", "rsg_stream") else (
            None if name == "rsg_default_options" else (C.c_longlong if name in ("rsg_submit", "rsg_submit_view") else
                                                         (C.c_size_t if name == "rsg_request_bytes" else C.c_int)))
    _LIB = L
    return L


def last_error() -> str:
    return load().rsg_last_error().decode()


def check(code: int, allow_notconv: bool = True) -> int:
    if code < 0 or (code > 0 and not allow_notconv):
        raise RsgError(code, last_error())
    return code


def ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None else None
