"""GB300 (sm_103a) implementation of generic-linalg's hot path, Python side.

The compute lives in ``libglinalg_gb300.so`` (CUDA kernels behind the C-ABI declared in
``include/glinalg.h``).  This module loads it with ctypes and mirrors the reference's
interface for the path:

* operator descriptors ``StaggeredU1Op`` (operators.h:7-15) and ``Stencil2D``
  (coarse_stencil.h:33-67);
* operator callbacks ``square_staggered_u1``, ``square_staggered_dagger_u1``,
  ``square_staggered_normal_u1``, ``square_laplace_u1``, ``apply_stencil_2d``,
  ``apply_stencil_2d_eo``, ``apply_stencil_2d_oe`` and the even/odd pieces
  ``square_staggered_deo_u1``, ``square_staggered_doe_u1``, ``square_staggered_m2mdeodoe_u1``,
  ``apply_square_staggered_m2mdeodoe_stencil`` with the reference's
  ``matrix_vector(lhs, rhs, extra)`` convention;
* the even/odd steps ``square_staggered_eoprec_prepare`` / ``_reconstruct`` and their stencil
  forms (operators.cpp:543-620, operators_stencil.cpp:179-236);
* solvers ``minv_vector_cg``, ``minv_vector_cg_restart``, ``minv_vector_cg_m``,
  ``minv_vector_bicgstab``, ``minv_vector_bicgstab_restart``, ``minv_vector_gcr``,
  ``minv_vector_gcr_restart`` and the siblings ``minv_vector_cr``, ``minv_vector_cr_restart``,
  ``minv_vector_minres``, ``minv_vector_cr_m``, ``minv_vector_bicgstab_l``,
  ``minv_vector_bicgstab_l_restart``, ``minv_vector_bicgstab_m``,
  ``minv_vector_cg_flex_precond``, ``minv_vector_gcr_var_precond`` (and their restarted forms,
  with ``identity_preconditioner``, ``minres_preconditioner``, ``gcr_preconditioner``) with the
  reference's argument order, returning ``InversionInfo`` (inverter_struct.h:14-43);
* ``InversionVerboseStruct`` and the ``VERB_*`` levels (verbosity.h:9-24);
* the U(1) gauge-field utilities of u1_utils.h: ``read_gauge_u1``, ``write_gauge_u1``,
  ``unit_gauge_u1``, ``get_plaquette_u1``, ``get_topo_u1``, ``apply_gauge_trans_u1``,
  ``apply_ape_smear_u1`` and ``Generator.rand_trans_u1``.

Fields are numpy complex128 arrays (host) or CUDA torch tensors of dtype complex128
(device; the call then passes device pointers).  As in the reference, the solver recognises
the operator by the callback it is given and the descriptor in ``extra_info``; any other
callback raises ``UnsupportedOperator`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _capi
from ._capi import (GLINALG_PTR_DEVICE, GLINALG_PTR_HOST, PREC_BFLOAT, PREC_DOUBLE, PREC_HALF,
                    PREC_SINGLE, GlinalgError, InfoStruct, OpDesc, SolverParams, VerbStruct, lib,
                    load_library)

__all__ = [
    "lib", "load_library", "GlinalgError", "UnsupportedOperator", "SolveTimeout",
    "GLINALG_SOLVE_CONVERGED", "GLINALG_SOLVE_MAX_ITER", "GLINALG_SOLVE_BREAKDOWN",
    "GLINALG_SOLVE_NONFINITE", "GLINALG_SOLVE_TIMEOUT",
    "StaggeredU1Op", "Stencil2D", "Operator", "InversionInfo", "InversionVerboseStruct",
    "VERB_PASS_THROUGH", "VERB_NONE", "VERB_SUMMARY", "VERB_RESTART_DETAIL", "VERB_DETAIL",
    "square_staggered_u1", "square_staggered_dagger_u1", "square_staggered_normal_u1",
    "square_laplace_u1", "apply_stencil_2d", "apply_stencil_2d_eo", "apply_stencil_2d_oe",
    "get_square_staggered_u1_stencil", "get_square_staggered_dagger_u1_stencil",
    "square_staggered_deo_u1", "square_staggered_doe_u1", "square_staggered_m2mdeodoe_u1",
    "apply_square_staggered_m2mdeodoe_stencil", "square_staggered_eoprec_prepare",
    "square_staggered_eoprec_reconstruct", "apply_square_staggered_eoprec_prepare_stencil",
    "apply_square_staggered_eoprec_reconstruct_stencil",
    "apply_stencil_2d_tb", "apply_stencil_2d_bt", "apply_square_staggered_m2mdtbdbt_stencil",
    "apply_square_staggered_normal_eo_stencil", "apply_square_staggered_normal_tb_stencil",
    "apply_square_staggered_dagger_eo_stencil", "apply_square_staggered_dagger_tb_stencil",
    "apply_square_staggered_tbprec_prepare_stencil", "apply_square_staggered_tbprec_reconstruct_stencil",
    "MgLevel", "block_normalize", "block_orthonormalize", "prolong", "restrict",
    "generate_coarse_from_fine_stencil", "MgPrecondStruct", "mg_preconditioner",
    "MINV_INVALID", "MINV_CG", "MINV_CR", "MINV_GCR", "MINV_BICGSTAB", "MINV_BICGSTAB_L", "MINV_MINRES",
    "NONE", "MINRES", "CG", "GCR", "BICGSTAB", "CR", "BICGSTAB_L", "MLEVEL_SMOOTH", "MLEVEL_RECURSIVE",
    "minv_vector_cg", "minv_vector_cg_restart", "minv_vector_cg_m", "minv_vector_bicgstab",
    "minv_vector_bicgstab_restart", "minv_vector_gcr", "minv_vector_gcr_restart",
    "minv_vector_cr", "minv_vector_cr_restart", "minv_vector_minres", "minv_vector_cr_m",
    "minv_vector_bicgstab_l", "minv_vector_bicgstab_l_restart", "minv_vector_bicgstab_m",
    "minv_vector_cg_flex_precond", "minv_vector_cg_flex_precond_restart",
    "minv_vector_gcr_var_precond", "minv_vector_gcr_var_precond_restart",
    "identity_preconditioner", "minres_preconditioner", "gcr_preconditioner",
    "MinresPrecondStruct", "GcrPrecondStruct",
    "Generator", "dot", "norm2sq", "staggered_force", "staggered_action_grad",
    "cg_batch", "cg_m_multi",
    "read_gauge_u1", "write_gauge_u1", "unit_gauge_u1", "get_plaquette_u1", "get_topo_u1",
    "apply_gauge_trans_u1", "apply_ape_smear_u1",
    "PREC_DOUBLE", "PREC_SINGLE", "PREC_HALF", "PREC_BFLOAT",
]

VERB_PASS_THROUGH, VERB_NONE, VERB_SUMMARY, VERB_RESTART_DETAIL, VERB_DETAIL = -1, 0, 1, 2, 3
# glinalg_solve_status (glinalg_info.status)
(GLINALG_SOLVE_CONVERGED, GLINALG_SOLVE_MAX_ITER, GLINALG_SOLVE_BREAKDOWN, GLINALG_SOLVE_NONFINITE,
 GLINALG_SOLVE_TIMEOUT) = 0, 1, 2, 3, 4

KIND_STAGGERED, KIND_STAGGERED_DAGGER, KIND_STAGGERED_NORMAL, KIND_LAPLACE = 0, 1, 2, 3
KIND_STENCIL, KIND_STENCIL_EO, KIND_STENCIL_OE = 4, 5, 6
KIND_STAGGERED_DEO, KIND_STAGGERED_DOE, KIND_STAGGERED_M2MDEODOE, KIND_STENCIL_M2MDEODOE = 7, 8, 9, 10
KIND_STENCIL_TB, KIND_STENCIL_BT, KIND_STENCIL_M2MDTBDBT = 11, 12, 13
KIND_STENCIL_NORMAL_EO, KIND_STENCIL_NORMAL_TB, KIND_STENCIL_DAGGER_EO, KIND_STENCIL_DAGGER_TB = 14, 15, 16, 17
_STENCIL_KINDS = (KIND_STENCIL, KIND_STENCIL_EO, KIND_STENCIL_OE, KIND_STENCIL_M2MDEODOE, KIND_STENCIL_TB,
                  KIND_STENCIL_BT, KIND_STENCIL_M2MDTBDBT, KIND_STENCIL_NORMAL_EO, KIND_STENCIL_NORMAL_TB,
                  KIND_STENCIL_DAGGER_EO, KIND_STENCIL_DAGGER_TB)


class UnsupportedOperator(GlinalgError):
    pass


# ---------------------------------------------------------------- field plumbing

def release_memory():
    """glinalg_release_memory: hand the memory the library's pools keep between calls (the work
    vectors of finished calls) back to the device."""
    _capi.check(lib().glinalg_release_memory(), "release_memory")


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _field_ptr(a, writable=False):
    """(pointer, n_complex, device) for a complex128 numpy array or torch tensor."""
    if _is_torch(a):
        import torch
        if a.dtype != torch.complex128 or not a.is_contiguous():
            raise TypeError("torch fields must be contiguous complex128 tensors")
        return C.c_void_p(a.data_ptr()), a.numel(), a.is_cuda
    if not isinstance(a, np.ndarray) or a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("numpy fields must be C-contiguous complex128 arrays")
    if writable and not a.flags["WRITEABLE"]:
        raise TypeError("output array is read-only")
    return C.c_void_p(a.ctypes.data), a.size, False


def _dptr(p):
    return C.cast(p, C.POINTER(C.c_double))


def _need(name, n, want):
    """The library gets plain pointers and reads (or writes) `want` values through them: refuse
    a shorter array here rather than let it run past the end."""
    if n < want:
        raise ValueError(f"{name} holds {n} values; this call needs {want}")


def _same_side(*devs):
    if len(set(devs)) > 1:
        raise ValueError("the arrays of one call must all be on the host or all on the device")


# ---------------------------------------------------------------- operator descriptors

class StaggeredU1Op:
    """Mirror of staggered_u1_op (operators.h:7-15)."""

    def __init__(self, lattice, mass, x_fine, y_fine, Nc=1, wilson_coeff=0.0):
        self.lattice = np.ascontiguousarray(lattice, dtype=np.complex128) if not _is_torch(lattice) else lattice
        self.mass = float(mass)
        self.x_fine, self.y_fine = int(x_fine), int(y_fine)
        self.Nc = int(Nc)
        self.wilson_coeff = float(wilson_coeff)


class Stencil2D:
    """Mirror of stencil_2d (coarse_stencil.h:33-67) on an lx x ly lattice with nc colours.
    stencil_size 2 allocates the two-link term."""

    def __init__(self, lx, ly, nc, stencil_size=1, shift=0j, eo_shift=0j, dof_shift=0j):
        self.lx, self.ly, self.nc = int(lx), int(ly), int(nc)
        v = self.lx * self.ly * self.nc * self.nc
        self.clover = np.zeros(v, np.complex128)
        self.hopping = np.zeros(4 * v, np.complex128)
        self.has_two = stencil_size == 2
        self.two_link = np.zeros(8 * v, np.complex128) if self.has_two else None
        self.shift, self.eo_shift, self.dof_shift = complex(shift), complex(eo_shift), complex(dof_shift)
        self.generated = False


class Operator:
    """A device-resident operator (glinalg_operator): links or stencil coefficients are copied
    to the GPU once; apply / solve calls then reuse them."""

    def __init__(self, kind, lx, ly, mass=0.0, links=None, nc=1, clover=None, hopping=None,
                 two_link=None, shift=0j, eo_shift=0j, dof_shift=0j):
        d = OpDesc()
        d.kind, d.lx, d.ly, d.nc, d.mass = int(kind), int(lx), int(ly), int(nc), float(mass)
        keep = []
        dev_flags = []
        # complex values glinalg_operator_create reads from each array: it gets plain pointers
        # and cannot check their lengths, so a short array is refused here instead of read past
        v = max(int(lx), 0) * max(int(ly), 0)
        nc2 = max(int(nc), 0) ** 2
        need = {"links": 2 * v, "clover": v * nc2, "hopping": 4 * v * nc2, "two_link": 8 * v * nc2}

        def put(name, a):
            if a is None:
                return
            a = a if _is_torch(a) else np.ascontiguousarray(a, dtype=np.complex128)
            p, n, dev = _field_ptr(a)
            if n < need[name]:
                raise ValueError(f"{name} holds {n} complex values; a {lx}x{ly} operator with nc = {nc} "
                                 f"reads {need[name]}")
            keep.append(a)
            dev_flags.append(dev)
            setattr(d, name, _dptr(p))

        put("links", links)
        put("clover", clover)
        put("hopping", hopping)
        put("two_link", two_link)
        for nm, z in (("shift", shift), ("eo_shift", eo_shift), ("dof_shift", dof_shift)):
            z = complex(z)
            getattr(d, nm)[0], getattr(d, nm)[1] = z.real, z.imag
        if dev_flags and all(dev_flags):
            d.flags = GLINALG_PTR_DEVICE
        elif any(dev_flags):
            raise TypeError("operator arrays must all be on the host or all on the device")
        h = C.c_void_p()
        _capi.check(lib().glinalg_operator_create(C.byref(d), C.byref(h)), "glinalg_operator_create")
        self.handle = h
        self.kind, self.lx, self.ly, self.nc = int(kind), int(lx), int(ly), int(nc)

    @property
    def size(self):
        return int(lib().glinalg_operator_size(self.handle))

    def set_mass(self, mass):
        _capi.check(lib().glinalg_operator_set_mass(self.handle, float(mass)), "set_mass")

    def apply(self, lhs, rhs):
        lp, ln, ldev = _field_ptr(lhs, writable=True)
        rp, rn, rdev = _field_ptr(rhs)
        if ln != self.size or rn != self.size or ldev != rdev:
            raise ValueError("field sizes/devices do not match the operator")
        _capi.check(lib().glinalg_operator_apply(self.handle, _dptr(lp), _dptr(rp),
                                                 GLINALG_PTR_DEVICE if ldev else 0), "apply")
        return lhs

    def close(self):
        if getattr(self, "handle", None):
            lib().glinalg_operator_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- reference-named callbacks

def _op_for(kind, extra):
    if isinstance(extra, Operator):
        return extra, False
    if kind in _STENCIL_KINDS:
        if not isinstance(extra, Stencil2D):
            raise UnsupportedOperator("stencil callbacks need a Stencil2D extra_info")
        return Operator(kind, extra.lx, extra.ly, nc=extra.nc, clover=extra.clover,
                        hopping=extra.hopping, two_link=extra.two_link, shift=extra.shift,
                        eo_shift=extra.eo_shift, dof_shift=extra.dof_shift), True
    if not isinstance(extra, StaggeredU1Op):
        raise UnsupportedOperator("U(1) callbacks need a StaggeredU1Op extra_info")
    return Operator(kind, extra.x_fine, extra.y_fine, mass=extra.mass, links=extra.lattice), True


def _callback(kind, name, ref):
    def cb(lhs, rhs, extra_data):
        op, temp = _op_for(kind, extra_data)
        try:
            op.apply(lhs, rhs)
        finally:
            if temp:
                op.close()
    cb.__name__ = name
    cb.__doc__ = f"lhs = A rhs on the GPU; replaces {name} ({ref})."
    cb._glinalg_kind = kind
    return cb


square_staggered_u1 = _callback(KIND_STAGGERED, "square_staggered_u1", "operators.cpp:184")
square_staggered_dagger_u1 = _callback(KIND_STAGGERED_DAGGER, "square_staggered_dagger_u1", "operators.cpp:372")
square_staggered_normal_u1 = _callback(KIND_STAGGERED_NORMAL, "square_staggered_normal_u1", "operators.cpp:444")
square_laplace_u1 = _callback(KIND_LAPLACE, "square_laplace_u1", "operators.cpp:73")
apply_stencil_2d = _callback(KIND_STENCIL, "apply_stencil_2d", "coarse_stencil.cpp:12")
apply_stencil_2d_eo = _callback(KIND_STENCIL_EO, "apply_stencil_2d_eo", "coarse_stencil.cpp:395")
apply_stencil_2d_oe = _callback(KIND_STENCIL_OE, "apply_stencil_2d_oe", "coarse_stencil.cpp:560")
square_staggered_deo_u1 = _callback(KIND_STAGGERED_DEO, "square_staggered_deo_u1", "operators.cpp:455")
square_staggered_doe_u1 = _callback(KIND_STAGGERED_DOE, "square_staggered_doe_u1", "operators.cpp:499")
square_staggered_m2mdeodoe_u1 = _callback(KIND_STAGGERED_M2MDEODOE, "square_staggered_m2mdeodoe_u1",
                                          "operators.cpp:566")
apply_square_staggered_m2mdeodoe_stencil = _callback(KIND_STENCIL_M2MDEODOE, "apply_square_staggered_m2mdeodoe_stencil",
                                                     "operators_stencil.cpp:197")
apply_stencil_2d_tb = _callback(KIND_STENCIL_TB, "apply_stencil_2d_tb", "coarse_stencil.cpp:725")
apply_stencil_2d_bt = _callback(KIND_STENCIL_BT, "apply_stencil_2d_bt", "coarse_stencil.cpp:1120")
apply_square_staggered_m2mdtbdbt_stencil = _callback(KIND_STENCIL_M2MDTBDBT, "apply_square_staggered_m2mdtbdbt_stencil",
                                                     "mg_complex.cpp:1228")
apply_square_staggered_normal_eo_stencil = _callback(KIND_STENCIL_NORMAL_EO, "apply_square_staggered_normal_eo_stencil",
                                                     "mg_complex.cpp:1277")
apply_square_staggered_normal_tb_stencil = _callback(KIND_STENCIL_NORMAL_TB, "apply_square_staggered_normal_tb_stencil",
                                                     "mg_complex.cpp:1305")
apply_square_staggered_dagger_eo_stencil = _callback(KIND_STENCIL_DAGGER_EO, "apply_square_staggered_dagger_eo_stencil",
                                                     "mg_complex.cpp:1335")
apply_square_staggered_dagger_tb_stencil = _callback(KIND_STENCIL_DAGGER_TB, "apply_square_staggered_dagger_tb_stencil",
                                                     "mg_complex.cpp:1355")


def _eo_step(kind, out, a, b, extra):
    op, temp = _op_for(kind, extra)
    try:
        if op.kind not in (KIND_STAGGERED_M2MDEODOE, KIND_STENCIL_M2MDEODOE, KIND_STENCIL_M2MDTBDBT):
            raise UnsupportedOperator("even/odd steps need an m^2 - D_eo D_oe operator")
        op_, on, odev = _field_ptr(out, writable=True)
        ap, an, adev = _field_ptr(a)
        n = op.size
        if on != n or an != n or adev != odev:
            raise ValueError("field sizes/devices do not match the operator")
        flags = GLINALG_PTR_DEVICE if odev else 0
        if b is None:
            _capi.check(lib().glinalg_eoprec_prepare(op.handle, _dptr(op_), _dptr(ap), flags), "eoprec_prepare")
        else:
            bp, bn, bdev = _field_ptr(b)
            if bn != n or bdev != odev:
                raise ValueError("field sizes/devices do not match the operator")
            _capi.check(lib().glinalg_eoprec_reconstruct(op.handle, _dptr(op_), _dptr(ap), _dptr(bp), flags),
                        "eoprec_reconstruct")
    finally:
        if temp:
            op.close()
    return out


def square_staggered_eoprec_prepare(rhs_e, rhs_orig, extra_data):
    """rhs_e = m rhs - D_eo rhs on even sites, 0 on odd sites (operators.cpp:543)."""
    return _eo_step(KIND_STAGGERED_M2MDEODOE, rhs_e, rhs_orig, None, extra_data)


def square_staggered_eoprec_reconstruct(lhs_full, lhs_e, rhs_o, extra_data):
    """lhs_full = lhs_e on even sites, (rhs_o - D_oe lhs_e) / m on odd sites (operators.cpp:592)."""
    return _eo_step(KIND_STAGGERED_M2MDEODOE, lhs_full, lhs_e, rhs_o, extra_data)


def apply_square_staggered_eoprec_prepare_stencil(rhs_e, rhs_orig, stenc):
    """The stencil form of square_staggered_eoprec_prepare (operators_stencil.cpp:181)."""
    return _eo_step(KIND_STENCIL_M2MDEODOE, rhs_e, rhs_orig, None, stenc)


def apply_square_staggered_eoprec_reconstruct_stencil(lhs_full, lhs_e, rhs_o, stenc):
    """The stencil form of square_staggered_eoprec_reconstruct (operators_stencil.cpp:220)."""
    return _eo_step(KIND_STENCIL_M2MDEODOE, lhs_full, lhs_e, rhs_o, stenc)


def apply_square_staggered_tbprec_prepare_stencil(rhs_t, rhs_orig, stenc):
    """rhs_t = m rhs - D_tb rhs on the top colours, 0 on the bottom ones (mg_complex.cpp:1211)."""
    return _eo_step(KIND_STENCIL_M2MDTBDBT, rhs_t, rhs_orig, None, stenc)


def apply_square_staggered_tbprec_reconstruct_stencil(lhs_full, lhs_t, rhs_b, stenc):
    """lhs_full = lhs_t on the top colours, (rhs_b - D_bt lhs_t) / Re(m) on the bottom ones
    (mg_complex.cpp:1252)."""
    return _eo_step(KIND_STENCIL_M2MDTBDBT, lhs_full, lhs_t, rhs_b, stenc)


def _stencil_builder(dagger):
    def build(stenc: Stencil2D, stagif: StaggeredU1Op):
        """Fills stenc's hopping terms from staggered links (operators_stencil.cpp:14-63 /
        :120-169); no-op if already generated or nc != 1, like the reference."""
        if stenc.generated or stenc.nc != 1:
            return
        sh = np.zeros(2)
        _capi.check(lib().glinalg_staggered_stencil(
            _dptr(_field_ptr(stagif.lattice)[0]), stenc.lx, stenc.ly, stagif.mass, int(dagger),
            _dptr(C.c_void_p(stenc.hopping.ctypes.data)), sh.ctypes.data_as(C.POINTER(C.c_double)), 0),
            "glinalg_staggered_stencil")
        stenc.shift, stenc.eo_shift, stenc.dof_shift = complex(sh[0], sh[1]), 0j, 0j
        stenc.generated = True
    return build


get_square_staggered_u1_stencil = _stencil_builder(False)
get_square_staggered_dagger_u1_stencil = _stencil_builder(True)


# ---------------------------------------------------------------- solvers

class InversionVerboseStruct:
    """Mirror of inversion_verbose_struct (verbosity.h:18-24)."""

    def __init__(self, verbosity=VERB_NONE, verb_prefix="", precond_verbosity=VERB_NONE,
                 precond_verb_prefix=""):
        self.verbosity, self.verb_prefix = verbosity, verb_prefix
        self.precond_verbosity, self.precond_verb_prefix = precond_verbosity, precond_verb_prefix

    def struct(self):
        v = VerbStruct()
        self._b = (self.verb_prefix.encode(), self.precond_verb_prefix.encode())
        v.verbosity, v.verb_prefix = self.verbosity, self._b[0]
        v.precond_verbosity, v.precond_verb_prefix = self.precond_verbosity, self._b[1]
        return v


class InversionInfo:
    """Mirror of inversion_info (inverter_struct.h:14-43) plus device diagnostics."""

    def __init__(self, s: InfoStruct, resSqmrhs=None):
        self.resSq = s.resSq
        self.iter = s.iter
        self.success = bool(s.success)
        self.name = s.name.decode()
        self.ops_count = s.ops_count
        self.resSqmrhs = resSqmrhs
        self.n_rhs = s.n_rhs if resSqmrhs is not None else -1
        self.status = s.status
        self.reliable_updates = s.reliable_updates
        self.device_ms = s.device_ms
        self.gbytes = s.gbytes
        self.kernel_ms = s.kernel_ms
        self.kernel_gbytes = s.kernel_gbytes
        self.kernel_launches = s.kernel_launches

    def __repr__(self):
        return (f"InversionInfo(name={self.name!r}, iter={self.iter}, success={self.success}, "
                f"ops_count={self.ops_count}, resSq={self.resSq:.6g}, status={self.status})")


def _resolve(matrix_vector, extra_info):
    kind = getattr(matrix_vector, "_glinalg_kind", None)
    if kind is None:
        raise UnsupportedOperator(
            f"{getattr(matrix_vector, '__name__', matrix_vector)!r} is not one of the GPU operator "
            "callbacks; there is no CPU fallback")
    return _op_for(kind, extra_info)


def _params(precision=PREC_DOUBLE, delta=0.0, device=False, wait_limit_us=0):
    p = SolverParams()
    p.precision, p.delta, p.flags = int(precision), float(delta), GLINALG_PTR_DEVICE if device else 0
    p.wait_limit_us = int(wait_limit_us)
    return p


class SolveTimeout(GlinalgError):
    """A bounded device-side wait of the solve gave up (info.status == GLINALG_SOLVE_TIMEOUT);
    the device is still usable.  `info` holds the solve's state when it stopped."""

    def __init__(self, msg, info):
        super().__init__(msg)
        self.info = info


def _solve(fn, phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity, restart=None,
           precision=PREC_DOUBLE, delta=0.0, extra_args=(), wait_limit_us=0):
    op, temp = _resolve(matrix_vector, extra_info)
    try:
        pp, pn, pdev = _field_ptr(phi, writable=True)
        bp, bn, bdev = _field_ptr(phi0)
        if pdev != bdev:
            raise ValueError("phi and phi0 must both be on the host or both on the device")
        if pn < size or bn < size:
            raise ValueError("fields are shorter than size")
        info = InfoStruct()
        verb = verbosity.struct() if verbosity is not None else None
        args = [op.handle, _dptr(pp), _dptr(bp), int(size), int(max_iter), float(eps)]
        if restart is not None:
            args.append(int(restart))
        args += list(extra_args)
        args += [C.byref(verb) if verb is not None else None,
                 C.byref(_params(precision, delta, pdev, wait_limit_us)), C.byref(info)]
        st = fn(*args)
        if st != 0 and info.status == GLINALG_SOLVE_TIMEOUT:
            raise SolveTimeout(f"{fn.__name__}: {lib().glinalg_last_error().decode()}", InversionInfo(info))
        _capi.check(st, fn.__name__)
        return InversionInfo(info)
    finally:
        if temp:
            op.close()


def minv_vector_cg(phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity=None,
                   precision=PREC_DOUBLE, delta=0.0, wait_limit_us=0):
    """minv_vector_cg (generic_cg.cpp:278).  precision != PREC_DOUBLE selects the mixed-precision
    CG with FP64 reliable updates (Hermitian operators only); wait_limit_us bounds its persistent
    kernels' waits for other blocks (glinalg_solver_params.wait_limit_us; a wait that runs out
    raises SolveTimeout)."""
    return _solve(lib().glinalg_cg, phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                  verbosity, precision=precision, delta=delta, wait_limit_us=wait_limit_us)


def minv_vector_cg_restart(phi, phi0, size, max_iter, eps, restart_freq, matrix_vector, extra_info,
                           verbosity=None):
    """minv_vector_cg_restart (generic_cg.cpp:387)."""
    return _solve(lib().glinalg_cg_restart, phi, phi0, size, max_iter, eps, matrix_vector,
                  extra_info, verbosity, restart=restart_freq)


def minv_vector_bicgstab(phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity=None):
    """minv_vector_bicgstab (generic_bicgstab.cpp:205)."""
    return _solve(lib().glinalg_bicgstab, phi, phi0, size, max_iter, eps, matrix_vector,
                  extra_info, verbosity)


def minv_vector_bicgstab_restart(phi, phi0, size, max_iter, eps, restart_freq, matrix_vector,
                                 extra_info, verbosity=None):
    """minv_vector_bicgstab_restart (generic_bicgstab.cpp:345)."""
    return _solve(lib().glinalg_bicgstab_restart, phi, phi0, size, max_iter, eps, matrix_vector,
                  extra_info, verbosity, restart=restart_freq)


def minv_vector_gcr(phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity=None):
    """minv_vector_gcr (generic_gcr.cpp:202)."""
    return _solve(lib().glinalg_gcr, phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                  verbosity)


def minv_vector_gcr_restart(phi, phi0, size, max_iter, eps, restart_freq, matrix_vector,
                            extra_info, verbosity=None):
    """minv_vector_gcr_restart (generic_gcr.cpp:337)."""
    return _solve(lib().glinalg_gcr_restart, phi, phi0, size, max_iter, eps, matrix_vector,
                  extra_info, verbosity, restart=restart_freq)


def minv_vector_cg_m(phi, phi0, n_shift, size, resid_freq_check, max_iter, eps, shifts,
                     matrix_vector, extra_info, worst_first=False, verbosity=None):
    """minv_vector_cg_m (generic_cg_m.cpp:312).  phi: a list of n_shift output fields."""
    return _multishift(lib().glinalg_cg_m, phi, phi0, n_shift, size, resid_freq_check, max_iter, eps,
                       shifts, matrix_vector, extra_info, worst_first, verbosity)


def minv_vector_cr_m(phi, phi0, n_shift, size, resid_freq_check, max_iter, eps, shifts,
                     matrix_vector, extra_info, worst_first=False, verbosity=None):
    """minv_vector_cr_m (generic_cr_m.cpp:323): multishift conjugate residual."""
    return _multishift(lib().glinalg_cr_m, phi, phi0, n_shift, size, resid_freq_check, max_iter, eps,
                       shifts, matrix_vector, extra_info, worst_first, verbosity)


def minv_vector_bicgstab_m(phi, phi0, n_shift, size, resid_freq_check, max_iter, eps, shifts,
                           matrix_vector, extra_info, worst_first=False, verbosity=None):
    """minv_vector_bicgstab_m (generic_bicgstab_m.cpp:402): multishift BiCGstab."""
    return _multishift(lib().glinalg_bicgstab_m, phi, phi0, n_shift, size, resid_freq_check, max_iter,
                       eps, shifts, matrix_vector, extra_info, worst_first, verbosity)


def minv_vector_cr(phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity=None):
    """minv_vector_cr (generic_cr.cpp:198)."""
    return _solve(lib().glinalg_cr, phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity)


def minv_vector_cr_restart(phi, phi0, size, max_iter, eps, restart_freq, matrix_vector, extra_info,
                           verbosity=None):
    """minv_vector_cr_restart (generic_cr.cpp:326)."""
    return _solve(lib().glinalg_cr_restart, phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                  verbosity, restart=restart_freq)


def minv_vector_minres(phi, phi0, size, max_iter, eps, *args, verbosity=None):
    """minv_vector_minres (generic_minres.cpp:130 and :234): the two reference overloads,
    ``(phi, phi0, size, max_iter, eps, omega, matrix_vector, extra_info[, verbosity])`` and
    ``(phi, phi0, size, max_iter, eps, matrix_vector, extra_info[, verbosity])`` (omega 1)."""
    if args and isinstance(args[0], (int, float)):
        omega, rest = float(args[0]), args[1:]
    else:
        omega, rest = 1.0, args
    matrix_vector, extra_info = rest[0], rest[1]
    if len(rest) > 2:
        verbosity = rest[2]
    return _solve(lib().glinalg_minres, phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                  verbosity, extra_args=(C.c_double(omega),))


def minv_vector_bicgstab_l(phi, phi0, size, max_iter, eps, l, matrix_vector, extra_info, verbosity=None):
    """minv_vector_bicgstab_l (generic_bicgstab_l.cpp:317)."""
    return _solve(lib().glinalg_bicgstab_l, phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                  verbosity, extra_args=(C.c_int(int(l)),))


def minv_vector_bicgstab_l_restart(phi, phi0, size, max_iter, eps, restart_freq, l, matrix_vector,
                                   extra_info, verbosity=None):
    """minv_vector_bicgstab_l_restart (generic_bicgstab_l.cpp:564)."""
    return _solve(lib().glinalg_bicgstab_l_restart, phi, phi0, size, max_iter, eps, matrix_vector,
                  extra_info, verbosity, restart=restart_freq, extra_args=(C.c_int(int(l)),))


class MinresPrecondStruct:
    """Mirror of minres_precond_struct_complex (generic_precond.h:37-43)."""

    def __init__(self, n_step, rel_res, matrix_vector, matrix_extra_data):
        self.n_step, self.rel_res = n_step, rel_res
        self.matrix_vector, self.matrix_extra_data = matrix_vector, matrix_extra_data


class GcrPrecondStruct(MinresPrecondStruct):
    """Mirror of gcr_precond_struct_complex (generic_precond.h:64-70)."""


def _precond(kind, name, ref):
    def pc(lhs, rhs, size, extra_data, verb=None):
        raise UnsupportedOperator(f"{name} runs inside the GPU solvers only; pass it to "
                                  "minv_vector_cg_flex_precond or minv_vector_gcr_var_precond")
    pc.__name__ = name
    pc.__doc__ = f"{name} ({ref}); selects the device preconditioner of the flexible solvers."
    pc._glinalg_precond = kind
    return pc


mg_preconditioner = _precond(3, "mg_preconditioner", "mg_complex.cpp:514")
identity_preconditioner = _precond(0, "identity_preconditioner", "generic_precond.cpp:34")
minres_preconditioner = _precond(1, "minres_preconditioner", "generic_precond.cpp:53")
gcr_preconditioner = _precond(2, "gcr_preconditioner", "generic_precond.cpp:70")


def _flex(fn, phi, phi0, size, max_iter, eps, restart, matrix_vector, extra_info, precond_matrix_vector,
          precond_info, verbosity):
    kind = getattr(precond_matrix_vector, "_glinalg_precond", None)
    if kind is None:
        raise UnsupportedOperator(f"{precond_matrix_vector!r} is not one of the GPU preconditioners")
    pc = _capi.PrecondStruct()
    pc.kind = kind
    pop, ptemp = None, False
    if kind == 3:
        pc.mg = precond_info.handle
    elif kind != 0:
        pc.n_step, pc.rel_res = int(precond_info.n_step), float(precond_info.rel_res)
        if precond_info.matrix_vector is not matrix_vector or precond_info.matrix_extra_data is not extra_info:
            pop, ptemp = _resolve(precond_info.matrix_vector, precond_info.matrix_extra_data)
            pc.op = pop.handle
    try:
        return _solve(fn, phi, phi0, size, max_iter, eps, matrix_vector, extra_info, verbosity,
                      restart=restart, extra_args=(C.byref(pc),))
    finally:
        if ptemp:
            pop.close()


def minv_vector_cg_flex_precond(phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                                precond_matrix_vector, precond_info, verbosity=None):
    """minv_vector_cg_flex_precond (generic_cg_flex_precond.cpp:223)."""
    return _flex(lib().glinalg_cg_flex_precond, phi, phi0, size, max_iter, eps, None, matrix_vector,
                 extra_info, precond_matrix_vector, precond_info, verbosity)


def minv_vector_cg_flex_precond_restart(phi, phi0, size, max_iter, eps, restart_freq, matrix_vector,
                                        extra_info, precond_matrix_vector, precond_info, verbosity=None):
    """minv_vector_cg_flex_precond_restart (generic_cg_flex_precond.cpp:367)."""
    return _flex(lib().glinalg_cg_flex_precond_restart, phi, phi0, size, max_iter, eps, restart_freq,
                 matrix_vector, extra_info, precond_matrix_vector, precond_info, verbosity)


def minv_vector_gcr_var_precond(phi, phi0, size, max_iter, eps, matrix_vector, extra_info,
                                precond_matrix_vector, precond_info, verbosity=None):
    """minv_vector_gcr_var_precond (generic_gcr_var_precond.cpp:220)."""
    return _flex(lib().glinalg_gcr_var_precond, phi, phi0, size, max_iter, eps, None, matrix_vector,
                 extra_info, precond_matrix_vector, precond_info, verbosity)


def minv_vector_gcr_var_precond_restart(phi, phi0, size, max_iter, eps, restart_freq, matrix_vector,
                                        extra_info, precond_matrix_vector, precond_info, verbosity=None):
    """minv_vector_gcr_var_precond_restart (generic_gcr_var_precond.cpp:369)."""
    return _flex(lib().glinalg_gcr_var_precond_restart, phi, phi0, size, max_iter, eps, restart_freq,
                 matrix_vector, extra_info, precond_matrix_vector, precond_info, verbosity)


def _multishift(fn, phi, phi0, n_shift, size, resid_freq_check, max_iter, eps, shifts,
                matrix_vector, extra_info, worst_first, verbosity):
    op, temp = _resolve(matrix_vector, extra_info)
    try:
        if len(phi) < n_shift:
            raise ValueError(f"phi holds {len(phi)} fields; n_shift is {n_shift}")
        ptrs = [_field_ptr(p, writable=True) for p in phi[:n_shift]]
        bp, bn, bdev = _field_ptr(phi0)
        if any(d != bdev for _, _, d in ptrs):
            raise ValueError("phi and phi0 must all be on the host or all on the device")
        for j, (_, n, _) in enumerate(ptrs):
            _need(f"phi[{j}]", n, size)
        _need("phi0", bn, size)
        arr = (C.POINTER(C.c_double) * n_shift)(*[_dptr(p) for p, _, _ in ptrs])
        sh = np.ascontiguousarray(shifts[:n_shift], dtype=np.float64)
        _need("shifts", sh.size, n_shift)
        res = np.zeros(n_shift)
        info = InfoStruct()
        info.resSqmrhs = res.ctypes.data_as(C.POINTER(C.c_double))
        info.n_rhs = n_shift
        verb = verbosity.struct() if verbosity is not None else None
        _capi.check(fn(op.handle, arr, _dptr(bp), int(n_shift), int(size),
                       int(resid_freq_check), int(max_iter), float(eps),
                       sh.ctypes.data_as(C.POINTER(C.c_double)), int(bool(worst_first)),
                       C.byref(verb) if verb is not None else None,
                       C.byref(_params(device=bdev)), C.byref(info)), fn.__name__)
        return InversionInfo(info, res)
    finally:
        if temp:
            op.close()


# ---------------------------------------------------------------- batched, force, BLAS, RNG

def cg_m_multi(op: Operator, phi, phi0, shifts, resid_freq_check=1, max_iter=10000, eps=1e-10,
               precision=PREC_DOUBLE):
    """Multishift CG for several sources at once.  phi: (n_rhs, n_shift, size), phi0:
    (n_rhs, size); both complex128, host or device.  precision PREC_SINGLE (staggered normal
    operator): an FP32 multishift with FP64 scalar recurrences, then every shifted system
    refined by the mixed CG to the FP64-true relative residual eps."""
    n_rhs, n_shift = phi.shape[0], phi.shape[1]
    pp, pn, dev = _field_ptr(phi, writable=True)
    bp, bn, bdev = _field_ptr(phi0)
    _same_side(dev, bdev)
    sh = np.ascontiguousarray(shifts, dtype=np.float64)
    _need("phi", pn, n_rhs * n_shift * op.size)
    _need("phi0", bn, n_rhs * op.size)
    _need("shifts", sh.size, n_shift)
    infos = (InfoStruct * n_rhs)()
    res = [np.zeros(n_shift) for _ in range(n_rhs)]
    for q in range(n_rhs):
        infos[q].resSqmrhs = res[q].ctypes.data_as(C.POINTER(C.c_double))
        infos[q].n_rhs = n_shift
    _capi.check(lib().glinalg_cg_m_multi(op.handle, _dptr(pp), _dptr(bp), n_rhs, n_shift, op.size,
                                         int(resid_freq_check), int(max_iter), float(eps),
                                         sh.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.byref(_params(precision, device=dev)), infos), "glinalg_cg_m_multi")
    return [InversionInfo(infos[q], res[q]) for q in range(n_rhs)]


def cg_batch(ops, phis, phi0s, max_iter=10000, eps=1e-10, precision=PREC_DOUBLE, delta=0.0):
    """CG on independent Hermitian systems (one Operator each)."""
    n = len(ops)
    if len(phis) != n or len(phi0s) != n:
        raise ValueError("one solution and one source field per operator")
    hs = (C.c_void_p * n)(*[o.handle.value for o in ops])
    pps = [_field_ptr(p, writable=True) for p in phis]
    bps = [_field_ptr(b) for b in phi0s]
    dev = pps[0][2]
    _same_side(*[d for _, _, d in pps + bps])
    for q in range(n):
        _need(f"phis[{q}]", pps[q][1], ops[q].size)
        _need(f"phi0s[{q}]", bps[q][1], ops[q].size)
    parr = (C.POINTER(C.c_double) * n)(*[_dptr(p) for p, _, _ in pps])
    barr = (C.POINTER(C.c_double) * n)(*[_dptr(p) for p, _, _ in bps])
    infos = (InfoStruct * n)()
    _capi.check(lib().glinalg_cg_batch(hs, n, parr, barr, int(max_iter), float(eps),
                                       C.byref(_params(precision, delta, dev)), infos), "glinalg_cg_batch")
    return [InversionInfo(infos[q]) for q in range(n)]


def staggered_force(op: Operator, X, Y, grad):
    """dS/dtheta = -2 Re(Y^dagger dM/dtheta X) for every link angle into grad (float64, 2V)."""
    xp, xn, dev = _field_ptr(X)
    yp, yn, ydev = _field_ptr(Y)
    if _is_torch(grad):
        import torch
        if grad.dtype != torch.float64 or not grad.is_contiguous():
            raise TypeError("grad must be a contiguous float64 tensor")
        gp, gn, gdev = C.c_void_p(grad.data_ptr()), grad.numel(), grad.is_cuda
    else:
        if grad.dtype != np.float64 or not grad.flags["C_CONTIGUOUS"] or not grad.flags["WRITEABLE"]:
            raise TypeError("grad must be a writable C-contiguous float64 array")
        gp, gn, gdev = C.c_void_p(grad.ctypes.data), grad.size, False
    _same_side(dev, ydev, gdev)
    _need("X", xn, op.size)
    _need("Y", yn, op.size)
    _need("grad", gn, 2 * op.size)
    _capi.check(lib().glinalg_staggered_force(op.handle, _dptr(xp), _dptr(yp), _dptr(gp),
                                              GLINALG_PTR_DEVICE if dev else 0), "glinalg_staggered_force")
    return grad


def staggered_action_grad(op: Operator, phi, sigma=0.0, eps=1e-12, max_iter=100000,
                          precision=PREC_DOUBLE, delta=0.0, X_out=None):
    """Returns (S, dS/dtheta, InversionInfo) for S = phi^dagger (D^dagger D + sigma)^-1 phi."""
    pp, n, dev = _field_ptr(phi)
    _need("phi", n, op.size)
    if X_out is not None:
        _need("X_out", _field_ptr(X_out, writable=True)[1], op.size)
        _same_side(dev, _field_ptr(X_out)[2])
    if dev:
        import torch
        grad = torch.zeros(2 * n, dtype=torch.float64, device=phi.device)
        gp = C.c_void_p(grad.data_ptr())
    else:
        grad = np.zeros(2 * n)
        gp = C.c_void_p(grad.ctypes.data)
    xo = _dptr(_field_ptr(X_out, writable=True)[0]) if X_out is not None else None
    act = C.c_double()
    info = InfoStruct()
    _capi.check(lib().glinalg_staggered_action_grad(op.handle, _dptr(pp), float(sigma), float(eps),
                                                    int(max_iter), C.byref(act), _dptr(gp), xo,
                                                    C.byref(_params(precision, delta, dev)), C.byref(info)),
                "glinalg_staggered_action_grad")
    return act.value, grad, InversionInfo(info)


def dot(a, b):
    """<a, b> = sum conj(a_i) b_i (generic_vector.h:102)."""
    ap, n, dev = _field_ptr(a)
    bp, bn, bdev = _field_ptr(b)
    _same_side(dev, bdev)
    _need("b", bn, n)
    out = (C.c_double * 2)()
    _capi.check(lib().glinalg_dot(_dptr(ap), _dptr(bp), n, out, GLINALG_PTR_DEVICE if dev else 0), "dot")
    return complex(out[0], out[1])


def norm2sq(a):
    """sum |a_i|^2 (generic_vector.h:132)."""
    ap, n, dev = _field_ptr(a)
    out = C.c_double()
    _capi.check(lib().glinalg_norm2sq(_dptr(ap), n, C.byref(out), GLINALG_PTR_DEVICE if dev else 0), "norm2sq")
    return out.value


class Generator:
    """One std::mt19937 stream as the reference's tests use it (``std::mt19937 generator(seed)``)."""

    def __init__(self, seed):
        self.h = C.c_void_p()
        _capi.check(lib().glinalg_rng_create(C.c_uint32(seed), C.byref(self.h)), "rng_create")

    def rand_gauge_u1(self, lx, ly):
        """rand_gauge_u1 (u1_utils.cpp:79-87)."""
        U = np.zeros(2 * lx * ly, np.complex128)
        _capi.check(lib().glinalg_rng_gauge_u1(self.h, _dptr(C.c_void_p(U.ctypes.data)), lx, ly), "gauge")
        return U

    def gauss_gauge_u1(self, lx, ly, beta):
        """gauss_gauge_u1 (u1_utils.cpp:92-112)."""
        U = np.zeros(2 * lx * ly, np.complex128)
        _capi.check(lib().glinalg_rng_gauss_gauge_u1(self.h, _dptr(C.c_void_p(U.ctypes.data)), lx, ly,
                                                     float(beta)), "gauss_gauge")
        return U

    def gaussian(self, n):
        """gaussian<complex> (generic_vector.h:48-60)."""
        v = np.zeros(n, np.complex128)
        _capi.check(lib().glinalg_rng_gaussian(self.h, _dptr(C.c_void_p(v.ctypes.data)), C.c_long(n)), "gaussian")
        return v

    def rand_trans_u1(self, lx, ly):
        """rand_trans_u1 (u1_utils.cpp:116-126): a random U(1) gauge transform."""
        g = np.zeros(lx * ly, np.complex128)
        _capi.check(lib().glinalg_rng_trans_u1(self.h, _dptr(C.c_void_p(g.ctypes.data)), lx, ly), "trans")
        return g

    def __del__(self):
        try:
            lib().glinalg_rng_destroy(self.h)
        except Exception:
            pass


# ---------------------------------------------------------------- U(1) gauge fields (u1_utils.h)

def _flags(dev):
    return GLINALG_PTR_DEVICE if dev else GLINALG_PTR_HOST


def read_gauge_u1(gauge_field, x_len, y_len, input_file):
    """read_gauge_u1 (u1_utils.cpp:17-38): fills the host array gauge_field from the
    reference's text format."""
    p, n, dev = _field_ptr(gauge_field, writable=True)
    if dev or n < 2 * x_len * y_len:
        raise ValueError("gauge_field must be a host array of 2*x_len*y_len entries")
    _capi.check(lib().glinalg_read_gauge_u1(_dptr(p), x_len, y_len, os.fsencode(input_file)), "read_gauge_u1")


def write_gauge_u1(gauge_field, x_len, y_len, output_file):
    """write_gauge_u1 (u1_utils.cpp:44-65)."""
    p, n, dev = _field_ptr(gauge_field)
    if dev or n < 2 * x_len * y_len:
        raise ValueError("gauge_field must be a host array of 2*x_len*y_len entries")
    _capi.check(lib().glinalg_write_gauge_u1(_dptr(p), x_len, y_len, os.fsencode(output_file)), "write_gauge_u1")


def unit_gauge_u1(gauge_field, x_len, y_len):
    """unit_gauge_u1 (u1_utils.cpp:69-75)."""
    p, n, dev = _field_ptr(gauge_field, writable=True)
    _need("gauge_field", n, 2 * x_len * y_len)
    _capi.check(lib().glinalg_unit_gauge_u1(_dptr(p), x_len, y_len, _flags(dev)), "unit_gauge_u1")


def get_plaquette_u1(gauge_field, x_len, y_len):
    """get_plaquette_u1 (u1_utils.cpp:190-207): the average plaquette (complex)."""
    p, n, dev = _field_ptr(gauge_field)
    _need("gauge_field", n, 2 * x_len * y_len)
    out = np.zeros(2)
    _capi.check(lib().glinalg_plaquette_u1(_dptr(p), x_len, y_len, out.ctypes.data_as(C.POINTER(C.c_double)),
                                           _flags(dev)), "plaquette_u1")
    return complex(out[0], out[1])


def get_topo_u1(gauge_field, x_len, y_len):
    """get_topo_u1 (u1_utils.cpp:210-226): the topological charge."""
    p, n, dev = _field_ptr(gauge_field)
    _need("gauge_field", n, 2 * x_len * y_len)
    out = C.c_double()
    _capi.check(lib().glinalg_topo_u1(_dptr(p), x_len, y_len, C.byref(out), _flags(dev)), "topo_u1")
    return out.value


def apply_gauge_trans_u1(gauge_field, gauge_trans, x_len, y_len):
    """apply_gauge_trans_u1 (u1_utils.cpp:128-142), in place."""
    p, n, dev = _field_ptr(gauge_field, writable=True)
    g, gn, gdev = _field_ptr(gauge_trans)
    if dev != gdev:
        raise ValueError("gauge_field and gauge_trans must both be on the host or both on the device")
    _need("gauge_field", n, 2 * x_len * y_len)
    _need("gauge_trans", gn, x_len * y_len)
    _capi.check(lib().glinalg_apply_gauge_trans_u1(_dptr(p), _dptr(g), x_len, y_len, _flags(dev)), "gauge_trans")


def apply_ape_smear_u1(smeared_field, gauge_field, x_len, y_len, alpha, n_iter):
    """apply_ape_smear_u1 (u1_utils.cpp:145-187)."""
    o, on, odev = _field_ptr(smeared_field, writable=True)
    p, n, dev = _field_ptr(gauge_field)
    if dev != odev:
        raise ValueError("both fields must be on the host or both on the device")
    _need("smeared_field", on, 2 * x_len * y_len)
    _need("gauge_field", n, 2 * x_len * y_len)
    _capi.check(lib().glinalg_apply_ape_smear_u1(_dptr(o), _dptr(p), x_len, y_len, float(alpha), int(n_iter),
                                                 _flags(dev)), "ape_smear_u1")


# ---------------------------------------------------------------- multigrid (mg_complex.cpp)

class MgLevel:
    """One level of mg_operator_struct_complex (mg_complex.h): a fine lattice x_fine x y_fine
    with nc_fine dof per site blocked blocksize_x x blocksize_y onto coarse sites with
    nc_coarse dof, and its null vectors (an (nc_coarse, x_fine*y_fine*nc_fine) complex array
    or list of fields), held on the device."""

    def __init__(self, x_fine, y_fine, nc_fine, blocksize_x, blocksize_y, nc_coarse, null_vectors):
        self.x_fine, self.y_fine, self.nc_fine = int(x_fine), int(y_fine), int(nc_fine)
        self.blocksize_x, self.blocksize_y, self.nc_coarse = int(blocksize_x), int(blocksize_y), int(nc_coarse)
        self.x_coarse, self.y_coarse = self.x_fine // self.blocksize_x, self.y_fine // self.blocksize_y
        self.fine_size = self.x_fine * self.y_fine * self.nc_fine
        self.coarse_size = self.x_coarse * self.y_coarse * self.nc_coarse
        if _is_torch(null_vectors):
            nv = null_vectors.contiguous()
            p, n, dev = _field_ptr(nv)
        else:
            nv = np.ascontiguousarray(np.asarray(null_vectors, dtype=np.complex128).reshape(-1))
            p, n, dev = _field_ptr(nv)
        if n != self.nc_coarse * self.fine_size:
            raise ValueError("null_vectors must hold nc_coarse fine fields")
        self.handle = C.c_void_p()
        _capi.check(lib().glinalg_mg_level_create(self.x_fine, self.y_fine, self.nc_fine, self.blocksize_x,
                                                  self.blocksize_y, self.nc_coarse, _dptr(p), _flags(dev),
                                                  C.byref(self.handle)), "mg_level_create")

    def null_vectors(self):
        out = np.zeros((self.nc_coarse, self.fine_size), np.complex128)
        _capi.check(lib().glinalg_mg_get_null_vectors(self.handle, _dptr(C.c_void_p(out.ctypes.data)), 0),
                    "mg_get_null_vectors")
        return out

    def __del__(self):
        try:
            if self.handle:
                lib().glinalg_mg_level_destroy(self.handle)
        except Exception:
            pass


def block_normalize(mgstruct: MgLevel):
    """block_normalize (mg_complex.cpp:191)."""
    _capi.check(lib().glinalg_mg_block_normalize(mgstruct.handle), "mg_block_normalize")


def block_orthonormalize(mgstruct: MgLevel):
    """block_orthonormalize (mg_complex.cpp:259)."""
    _capi.check(lib().glinalg_mg_block_orthonormalize(mgstruct.handle), "mg_block_orthonormalize")


def prolong(vec_fine, vec_coarse, mgstruct: MgLevel):
    """prolong (mg_complex.cpp:372): vec_fine = P vec_coarse."""
    o, no, d1 = _field_ptr(vec_fine, writable=True)
    i, ni, d2 = _field_ptr(vec_coarse)
    if d1 != d2 or no < mgstruct.fine_size or ni < mgstruct.coarse_size:
        raise ValueError("field sizes / devices do not match the level")
    _capi.check(lib().glinalg_mg_prolong(mgstruct.handle, _dptr(o), _dptr(i), _flags(d1)), "mg_prolong")


def restrict(vec_coarse, vec_fine, mgstruct: MgLevel):
    """restrict (mg_complex.cpp:421): vec_coarse = P^dagger vec_fine."""
    o, no, d1 = _field_ptr(vec_coarse, writable=True)
    i, ni, d2 = _field_ptr(vec_fine)
    if d1 != d2 or no < mgstruct.coarse_size or ni < mgstruct.fine_size:
        raise ValueError("field sizes / devices do not match the level")
    _capi.check(lib().glinalg_mg_restrict(mgstruct.handle, _dptr(o), _dptr(i), _flags(d1)), "mg_restrict")


def _coarse_operator(op_handle, mgstruct):
    """Wraps a library-created coarse stencil operator."""
    c = Operator.__new__(Operator)
    c.handle = op_handle
    c.kind, c.lx, c.ly, c.nc = KIND_STENCIL, mgstruct.x_coarse, mgstruct.y_coarse, mgstruct.nc_coarse
    return c


def generate_coarse_from_fine_stencil(stenc_coarse, stenc_fine, mgstruct: MgLevel, ignore_shifts=False):
    """generate_coarse_from_fine_stencil (mg_complex.cpp:827): the Galerkin coarse stencil
    P^dagger A P.  stenc_fine: a Stencil2D or a stencil Operator; stenc_coarse: a Stencil2D
    whose clover and hopping arrays receive the coarse coefficients, or None.  Returns the
    coarse operator on the device (a stencil Operator)."""
    fine, temp = (stenc_fine, False) if isinstance(stenc_fine, Operator) else _op_for(KIND_STENCIL, stenc_fine)
    try:
        h = C.c_void_p()
        _capi.check(lib().glinalg_mg_coarse_stencil(mgstruct.handle, fine.handle, int(bool(ignore_shifts)),
                                                    C.byref(h)), "mg_coarse_stencil")
        coarse = _coarse_operator(h, mgstruct)
    finally:
        if temp:
            fine.close()
    if stenc_coarse is not None:
        # the library writes the coarse clover (V_c nc_c^2) and hopping (4 V_c nc_c^2) terms
        cc = mgstruct.coarse_size * mgstruct.nc_coarse
        _need("stenc_coarse.clover", stenc_coarse.clover.size, cc)
        _need("stenc_coarse.hopping", stenc_coarse.hopping.size, 4 * cc)
        _capi.check(lib().glinalg_operator_stencil_get(coarse.handle, _dptr(C.c_void_p(stenc_coarse.clover.ctypes.data)),
                                                       _dptr(C.c_void_p(stenc_coarse.hopping.ctypes.data)), 0),
                    "operator_stencil_get")
        stenc_coarse.generated = True
    return coarse


# minv_inverter (generic_inverters.h:70-81), inner_solver (mg.h:5-14), mg_multilevel_type
MINV_INVALID, MINV_CG, MINV_CR, MINV_GCR, MINV_BICGSTAB, MINV_BICGSTAB_L, MINV_MINRES = -1, 0, 1, 2, 3, 4, 7
NONE, MINRES, CG, GCR, BICGSTAB, CR, BICGSTAB_L = 0, 1, 2, 3, 4, 5, 6
MLEVEL_SMOOTH, MLEVEL_RECURSIVE = 0, 1


class MgPrecondStruct:
    """Mirror of mg_precond_struct_complex (mg_complex.h) over a device hierarchy: ops[0] the
    fine operator, ops[l+1] the coarse operator of levels[l] (MgLevel).  Pass it as the
    precond_info of mg_preconditioner to minv_vector_cg_flex_precond /
    minv_vector_gcr_var_precond, or call apply(lhs, rhs)."""

    def __init__(self, ops, levels, in_smooth_type=MINV_MINRES, omega_smooth=1.0, n_pre_smooth=None,
                 n_post_smooth=None, normal_eqn_mg=False, normal_eqn_smooth=False, mlevel_type=MLEVEL_SMOOTH,
                 in_solve_type=GCR, n_max=64, n_restart=32, rel_res=None):
        nr = len(levels)
        if len(ops) != nr + 1:
            raise ValueError("need one more operator than levels")
        p = _capi.MgParams()
        p.smoother, p.omega_smooth = int(in_smooth_type), float(omega_smooth)
        for l in range(nr):
            p.n_pre_smooth[l] = int((n_pre_smooth or [0] * nr)[l])
            p.n_post_smooth[l] = int((n_post_smooth or [0] * nr)[l])
            p.rel_res[l] = float((rel_res or [1e-1] * nr)[l])
        p.normal_eqn_mg, p.normal_eqn_smooth = int(normal_eqn_mg), int(normal_eqn_smooth)
        p.mlevel_type, p.coarse_solver = int(mlevel_type), int(in_solve_type)
        p.n_max, p.n_restart = int(n_max), int(n_restart)
        self.ops, self.levels = list(ops), list(levels)
        oa = (C.c_void_p * (nr + 1))(*[o.handle.value for o in self.ops])
        la = (C.c_void_p * nr)(*[lv.handle.value for lv in self.levels])
        self.handle = C.c_void_p()
        _capi.check(lib().glinalg_mg_create(nr, oa, la, C.byref(p), C.byref(self.handle)), "mg_create")

    def apply(self, lhs, rhs):
        """One application of mg_preconditioner on the finest level."""
        o, no, d1 = _field_ptr(lhs, writable=True)
        i, ni, d2 = _field_ptr(rhs)
        if d1 != d2:
            raise ValueError("lhs and rhs must both be on the host or both on the device")
        _need("lhs", no, self.ops[0].size)
        _need("rhs", ni, self.ops[0].size)
        _capi.check(lib().glinalg_mg_apply(self.handle, _dptr(o), _dptr(i), _flags(d1)), "mg_apply")

    def __del__(self):
        try:
            if self.handle:
                lib().glinalg_mg_destroy(self.handle)
        except Exception:
            pass
