"""ctypes declarations of the C-ABI in include/glinalg.h and the library loader.

The library is the in-tree ``libglinalg_gb300.so`` built by ``build.py``.  Loading fails
loudly when it is missing: there is no CPU implementation to fall back to.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libglinalg_gb300.so")

GLINALG_PTR_HOST, GLINALG_PTR_DEVICE = 0, 1
PREC_DOUBLE, PREC_SINGLE, PREC_HALF, PREC_BFLOAT = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)


class GlinalgError(RuntimeError):
    pass


class OpDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("lx", C.c_int), ("ly", C.c_int), ("nc", C.c_int),
                ("mass", C.c_double), ("links", _dp), ("clover", _dp), ("hopping", _dp),
                ("two_link", _dp), ("shift", C.c_double * 2), ("eo_shift", C.c_double * 2),
                ("dof_shift", C.c_double * 2), ("flags", C.c_int)]


class VerbStruct(C.Structure):
    _fields_ = [("verbosity", C.c_int), ("verb_prefix", C.c_char_p),
                ("precond_verbosity", C.c_int), ("precond_verb_prefix", C.c_char_p)]


class InfoStruct(C.Structure):
    _fields_ = [("resSq", C.c_double), ("iter", C.c_int), ("success", C.c_int),
                ("ops_count", C.c_int), ("name", C.c_char * 64), ("resSqmrhs", _dp),
                ("n_rhs", C.c_int), ("status", C.c_int), ("reliable_updates", C.c_int),
                ("device_ms", C.c_double), ("gbytes", C.c_double), ("kernel_ms", C.c_double),
                ("kernel_gbytes", C.c_double), ("kernel_launches", C.c_int)]


class SolverParams(C.Structure):
    _fields_ = [("precision", C.c_int), ("delta", C.c_double), ("flags", C.c_int),
                ("wait_limit_us", C.c_int)]


class PrecondStruct(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_step", C.c_int), ("rel_res", C.c_double), ("op", C.c_void_p),
                ("mg", C.c_void_p)]


MG_MAX_LEVELS = 8


class MgParams(C.Structure):
    _fields_ = [("smoother", C.c_int), ("omega_smooth", C.c_double),
                ("n_pre_smooth", C.c_int * MG_MAX_LEVELS), ("n_post_smooth", C.c_int * MG_MAX_LEVELS),
                ("normal_eqn_mg", C.c_int), ("normal_eqn_smooth", C.c_int), ("mlevel_type", C.c_int),
                ("coarse_solver", C.c_int), ("n_max", C.c_int), ("n_restart", C.c_int),
                ("rel_res", C.c_double * MG_MAX_LEVELS)]


# Every function the header declares, with its ctypes prototype.
def _prototypes():
    P, vp, i, d, l, u32 = C.POINTER, C.c_void_p, C.c_int, C.c_double, C.c_long, C.c_uint32
    st = C.c_int
    solver = [vp, _dp, _dp, i, i, d, P(VerbStruct), P(SolverParams), P(InfoStruct)]
    restart = [vp, _dp, _dp, i, i, d, i, P(VerbStruct), P(SolverParams), P(InfoStruct)]
    return {
        "glinalg_abi_version": (i, []),
        "glinalg_status_string": (C.c_char_p, [st]),
        "glinalg_last_error": (C.c_char_p, []),
        "glinalg_device_count": (i, []),
        "glinalg_set_stream": (st, [vp, i]),
        "glinalg_release_memory": (st, []),
        "glinalg_profile_mixed_kernels": (st, [vp, i, i, _dp, _dp]),
        "glinalg_tuned_tile": (i, [vp, i]),
        "glinalg_tuned_persist": (i, [vp, i]),
        "glinalg_eoprec_prepare": (st, [vp, _dp, _dp, i]),
        "glinalg_eoprec_reconstruct": (st, [vp, _dp, _dp, _dp, i]),
        "glinalg_tbprec_prepare": (st, [vp, _dp, _dp, i]),
        "glinalg_mg_level_create": (st, [i, i, i, i, i, i, _dp, i, P(vp)]),
        "glinalg_mg_level_destroy": (st, [vp]),
        "glinalg_mg_get_null_vectors": (st, [vp, _dp, i]),
        "glinalg_mg_block_normalize": (st, [vp]),
        "glinalg_mg_block_orthonormalize": (st, [vp]),
        "glinalg_mg_prolong": (st, [vp, _dp, _dp, i]),
        "glinalg_mg_restrict": (st, [vp, _dp, _dp, i]),
        "glinalg_mg_coarse_stencil": (st, [vp, vp, i, P(vp)]),
        "glinalg_operator_stencil_get": (st, [vp, _dp, _dp, i]),
        "glinalg_mg_create": (st, [i, P(vp), P(vp), P(MgParams), P(vp)]),
        "glinalg_mg_destroy": (st, [vp]),
        "glinalg_mg_apply": (st, [vp, _dp, _dp, i]),
        "glinalg_tbprec_reconstruct": (st, [vp, _dp, _dp, _dp, i]),
        "glinalg_profile_persist_kernel": (st, [vp, i, i, i, _dp, _dp, P(i)]),
        "glinalg_probe_smem_bandwidth": (st, [_dp, _dp]),
        "glinalg_staggered_normal_apply_noalloc": (st, [_dp, d, i, i, _dp, _dp, vp]),
        "glinalg_operator_create": (st, [P(OpDesc), P(vp)]),
        "glinalg_operator_destroy": (st, [vp]),
        "glinalg_operator_set_mass": (st, [vp, d]),
        "glinalg_operator_size": (l, [vp]),
        "glinalg_operator_apply": (st, [vp, _dp, _dp, i]),
        "glinalg_staggered_stencil": (st, [_dp, i, i, d, i, _dp, _dp, i]),
        "glinalg_dot": (st, [_dp, _dp, l, _dp, i]),
        "glinalg_norm2sq": (st, [_dp, l, _dp, i]),
        "glinalg_cg": (st, solver),
        "glinalg_cg_restart": (st, restart),
        "glinalg_bicgstab": (st, solver),
        "glinalg_bicgstab_restart": (st, restart),
        "glinalg_gcr": (st, solver),
        "glinalg_gcr_restart": (st, restart),
        "glinalg_cg_m": (st, [vp, P(_dp), _dp, i, i, i, i, d, _dp, i, P(VerbStruct),
                              P(SolverParams), P(InfoStruct)]),
        "glinalg_cr": (st, solver),
        "glinalg_cr_restart": (st, restart),
        "glinalg_minres": (st, [vp, _dp, _dp, i, i, d, d, P(VerbStruct), P(SolverParams), P(InfoStruct)]),
        "glinalg_bicgstab_l": (st, [vp, _dp, _dp, i, i, d, i, P(VerbStruct), P(SolverParams), P(InfoStruct)]),
        "glinalg_bicgstab_l_restart": (st, [vp, _dp, _dp, i, i, d, i, i, P(VerbStruct), P(SolverParams),
                                            P(InfoStruct)]),
        "glinalg_cr_m": (st, [vp, P(_dp), _dp, i, i, i, i, d, _dp, i, P(VerbStruct),
                              P(SolverParams), P(InfoStruct)]),
        "glinalg_bicgstab_m": (st, [vp, P(_dp), _dp, i, i, i, i, d, _dp, i, P(VerbStruct),
                                    P(SolverParams), P(InfoStruct)]),
        "glinalg_cg_flex_precond": (st, [vp, _dp, _dp, i, i, d, P(PrecondStruct), P(VerbStruct),
                                         P(SolverParams), P(InfoStruct)]),
        "glinalg_cg_flex_precond_restart": (st, [vp, _dp, _dp, i, i, d, i, P(PrecondStruct), P(VerbStruct),
                                                 P(SolverParams), P(InfoStruct)]),
        "glinalg_gcr_var_precond": (st, [vp, _dp, _dp, i, i, d, P(PrecondStruct), P(VerbStruct),
                                         P(SolverParams), P(InfoStruct)]),
        "glinalg_gcr_var_precond_restart": (st, [vp, _dp, _dp, i, i, d, i, P(PrecondStruct), P(VerbStruct),
                                                 P(SolverParams), P(InfoStruct)]),
        "glinalg_cg_m_multi": (st, [vp, _dp, _dp, i, i, i, i, i, d, _dp, P(SolverParams),
                                    P(InfoStruct)]),
        "glinalg_cg_batch": (st, [P(vp), i, P(_dp), P(_dp), i, d, P(SolverParams), P(InfoStruct)]),
        "glinalg_staggered_force": (st, [vp, _dp, _dp, _dp, i]),
        "glinalg_staggered_action_grad": (st, [vp, _dp, d, d, i, _dp, _dp, _dp, P(SolverParams),
                                               P(InfoStruct)]),
        "glinalg_rng_create": (st, [u32, P(vp)]),
        "glinalg_rng_destroy": (st, [vp]),
        "glinalg_rng_gauge_u1": (st, [vp, _dp, i, i]),
        "glinalg_rng_gauss_gauge_u1": (st, [vp, _dp, i, i, d]),
        "glinalg_rng_gaussian": (st, [vp, _dp, l]),
        "glinalg_rng_trans_u1": (st, [vp, _dp, i, i]),
        "glinalg_read_gauge_u1": (st, [_dp, i, i, C.c_char_p]),
        "glinalg_write_gauge_u1": (st, [_dp, i, i, C.c_char_p]),
        "glinalg_unit_gauge_u1": (st, [_dp, i, i, i]),
        "glinalg_plaquette_u1": (st, [_dp, i, i, _dp, i]),
        "glinalg_topo_u1": (st, [_dp, i, i, _dp, i]),
        "glinalg_apply_gauge_trans_u1": (st, [_dp, _dp, i, i, i]),
        "glinalg_apply_ape_smear_u1": (st, [_dp, _dp, i, i, d, i, i]),
    }


PROTOTYPES = _prototypes()

_lock = threading.Lock()
_lib = None


def load_library(path=LIB_PATH):
    """Load the CUDA library (building nothing); raises GlinalgError if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise GlinalgError(
                f"{path} is missing: build it with `python generic-linalg_gb300/build.py` "
                "(there is no CPU fallback)")
        L = C.CDLL(path)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def lib():
    return _lib if _lib is not None else load_library()


def check(status, what):
    if status != 0:
        L = lib()
        msg = L.glinalg_status_string(status).decode()
        detail = L.glinalg_last_error().decode()
        raise GlinalgError(f"{what}: {msg} ({detail})")
