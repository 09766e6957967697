"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps oracle/_build/liboracle.so, the C99 restatement of the reference's
operators and solvers (oracle.c).  ``RefOracle`` wraps oracle/_ref/libref_oracle.so, the
reference's own sources compiled by ``make -C oracle ref``; it exists only where the
reference checkout is present and is used to pin the restatement and to write the golden
fixtures.  Only tests, the smoke check and the CPU-baseline leg of bench.py import this
module; the product never does.

Fields are numpy complex128 arrays (site i = y*lx + x); links are complex128 of length
2*lx*ly with U[2*i + mu].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_oracle.so")

KIND = {
    "staggered": 0,
    "staggered_dagger": 1,
    "staggered_normal": 2,
    "laplace": 3,
    "stencil": 4,
    "stencil_eo": 5,
    "stencil_oe": 6,
    "staggered_deo": 7,
    "staggered_doe": 8,
    "staggered_m2mdeodoe": 9,
    "stencil_m2mdeodoe": 10,
    "stencil_tb": 11,
    "stencil_bt": 12,
    "stencil_m2mdtbdbt": 13,
    "stencil_normal_eo": 14,
    "stencil_normal_tb": 15,
    "stencil_dagger_eo": 16,
    "stencil_dagger_tb": 17,
}

_dp = C.POINTER(C.c_double)


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


class OrcOp(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("lx", C.c_int), ("ly", C.c_int), ("nc", C.c_int),
        ("mass", C.c_double),
        ("links", _dp), ("clover", _dp), ("hopping", _dp), ("two_link", _dp),
        ("shift", C.c_double * 2), ("eo_shift", C.c_double * 2), ("dof_shift", C.c_double * 2),
    ]


class OrcInfo(C.Structure):
    _fields_ = [("resSq", C.c_double), ("iter", C.c_int), ("success", C.c_int),
                ("ops_count", C.c_int), ("name", C.c_char * 64)]

    def as_dict(self):
        return {"resSq": self.resSq, "iter": self.iter, "success": bool(self.success),
                "ops_count": self.ops_count, "name": self.name.decode()}


REF_RECORD = os.path.join(HERE, "_ref", "REFERENCE_DIR")


def reference_dir():
    """The reference checkout that the reference-compiled builds and fixture scripts read:
    GLINALG_REFERENCE_DIR if set, else the checkout the last reference build compiled from
    (recorded in oracle/_ref/REFERENCE_DIR), else None."""
    d = os.environ.get("GLINALG_REFERENCE_DIR")
    if d:
        return d
    try:
        with open(REF_RECORD) as f:
            d = f.read().strip()
        return d if os.path.isdir(d) else None
    except OSError:
        return None


def build(quiet=True, reference=None):
    """Compile liboracle.so, and libref_oracle.so when a reference checkout is given (the
    argument, else GLINALG_REFERENCE_DIR) and present."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=out)
    ref = reference or os.environ.get("GLINALG_REFERENCE_DIR")
    if ref and os.path.isdir(ref):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], stdout=out)
        with open(REF_RECORD, "w") as f:
            f.write(os.path.abspath(ref) + "\n")


PRECOND = {"identity": 0, "minres": 1, "gcr": 2}


class Generator:
    """The reference tests' input generators on one std::mt19937 stream (oracle/inputs.cpp):
    rand_gauge_u1, gauss_gauge_u1, rand_trans_u1 and gaussian, drawn in the reference's order."""

    def __init__(self, seed, path=LIB_PATH):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_rng_create.argtypes = [C.c_uint]
        L.orc_rng_create.restype = C.c_void_p
        L.orc_rng_destroy.argtypes = [C.c_void_p]
        L.orc_rng_gauge_u1.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int]
        L.orc_rng_gauss_gauge_u1.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, C.c_double]
        L.orc_rng_trans_u1.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int]
        L.orc_rng_gaussian.argtypes = [C.c_void_p, _dp, C.c_long]
        self.lib = L
        self.h = L.orc_rng_create(int(seed))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_rng_destroy(self.h)
            self.h = None

    def rand_gauge_u1(self, lx, ly):
        U = np.empty(2 * lx * ly, np.complex128)
        self.lib.orc_rng_gauge_u1(self.h, _ptr(U), lx, ly)
        return U

    def gauss_gauge_u1(self, lx, ly, beta):
        U = np.empty(2 * lx * ly, np.complex128)
        self.lib.orc_rng_gauss_gauge_u1(self.h, _ptr(U), lx, ly, beta)
        return U

    def rand_trans_u1(self, lx, ly):
        t = np.empty(lx * ly, np.complex128)
        self.lib.orc_rng_trans_u1(self.h, _ptr(t), lx, ly)
        return t

    def gaussian(self, n):
        v = np.empty(n, np.complex128)
        self.lib.orc_rng_gaussian(self.h, _ptr(v), n)
        return v


class OrcPrecond(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_step", C.c_int), ("rel_res", C.c_double),
                ("op", C.POINTER(OrcOp))]


class Operator:
    """Keeps the numpy arrays of one operator alive for the OrcOp that points at them."""

    def __init__(self, kind, lx, ly, mass=0.0, links=None, nc=1, clover=None, hopping=None,
                 two_link=None, shift=0j, eo_shift=0j, dof_shift=0j):
        self.kind = KIND[kind] if isinstance(kind, str) else int(kind)
        self.lx, self.ly, self.nc, self.mass = int(lx), int(ly), int(nc), float(mass)
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.complex128)
        self.links, self.clover, self.hopping, self.two_link = c(links), c(clover), c(hopping), c(two_link)
        self.shift, self.eo_shift, self.dof_shift = complex(shift), complex(eo_shift), complex(dof_shift)
        s = OrcOp()
        s.kind, s.lx, s.ly, s.nc, s.mass = self.kind, self.lx, self.ly, self.nc, self.mass
        s.links, s.clover = _ptr(self.links), _ptr(self.clover)
        s.hopping, s.two_link = _ptr(self.hopping), _ptr(self.two_link)
        for name in ("shift", "eo_shift", "dof_shift"):
            z = getattr(self, name)
            getattr(s, name)[0], getattr(s, name)[1] = z.real, z.imag
        self.struct = s

    @property
    def size(self):
        v = self.lx * self.ly
        return v * self.nc if (KIND["stencil"] <= self.kind <= KIND["stencil_oe"] or
                               self.kind >= KIND["stencil_tb"]) else v

    def shifts6(self):
        return np.array([self.shift.real, self.shift.imag, self.eo_shift.real,
                         self.eo_shift.imag, self.dof_shift.real, self.dof_shift.imag])


class OrcMgLevel(C.Structure):
    _fields_ = [("lx", C.c_int), ("ly", C.c_int), ("nc_f", C.c_int), ("bx", C.c_int), ("by", C.c_int),
                ("nc_c", C.c_int), ("null_vectors", _dp)]


class Oracle:
    def __init__(self, path=LIB_PATH):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        self.lib = L
        P = C.POINTER
        L.orc_apply.argtypes = [P(OrcOp), _dp, _dp]
        L.orc_staggered_stencil.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int]
        L.orc_dot.argtypes = [_dp, _dp, C.c_long, _dp]
        L.orc_norm2sq.argtypes = [_dp, C.c_long]
        L.orc_norm2sq.restype = C.c_double
        L.orc_diffnorm2sq.argtypes = [_dp, _dp, C.c_long]
        L.orc_diffnorm2sq.restype = C.c_double
        solver_args = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, P(OrcInfo), _dp, C.c_int]
        for n in ("orc_cg", "orc_bicgstab", "orc_gcr"):
            getattr(L, n).argtypes = solver_args
        for n in ("orc_cg_restart", "orc_bicgstab_restart", "orc_gcr_restart"):
            getattr(L, n).argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int, P(OrcInfo)]
        L.orc_cg_m.argtypes = [P(OrcOp), _dp, _dp, C.c_int, C.c_long, C.c_int, C.c_int, C.c_double,
                               _dp, C.c_int, P(OrcInfo), _dp, _dp, C.c_int]
        L.orc_staggered_force.argtypes = [_dp, C.c_double, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_cr.argtypes = solver_args
        L.orc_cr_restart.argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int, P(OrcInfo)]
        L.orc_minres.argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_double,
                                 P(OrcInfo), _dp, C.c_int]
        L.orc_bicgstab_l.argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                     P(OrcInfo), _dp, C.c_int]
        L.orc_bicgstab_l_restart.argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                             C.c_int, P(OrcInfo)]
        for n in ("orc_cr_m", "orc_bicgstab_m"):
            getattr(L, n).argtypes = L.orc_cg_m.argtypes
        for n in ("orc_fpcg", "orc_vpgcr"):
            getattr(L, n).argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, P(OrcPrecond),
                                      P(OrcInfo), _dp, C.c_int]
        for n in ("orc_fpcg_restart", "orc_vpgcr_restart"):
            getattr(L, n).argtypes = [P(OrcOp), _dp, _dp, C.c_long, C.c_int, C.c_double, C.c_int,
                                      P(OrcPrecond), P(OrcInfo)]
        L.orc_eoprec_prepare.argtypes = [P(OrcOp), _dp, _dp]
        L.orc_plaquette_u1.argtypes = [_dp, C.c_int, C.c_int, _dp]
        L.orc_tbprec_prepare.argtypes = [P(OrcOp), _dp, _dp]
        L.orc_tbprec_reconstruct.argtypes = [P(OrcOp), _dp, _dp, _dp]
        for n in ("orc_mg_block_normalize", "orc_mg_block_orthonormalize"):
            getattr(L, n).argtypes = [P(OrcMgLevel)]
        L.orc_mg_prolong.argtypes = [P(OrcMgLevel), _dp, _dp]
        L.orc_mg_restrict.argtypes = [P(OrcMgLevel), _dp, _dp]
        L.orc_mg_coarse_stencil.argtypes = [P(OrcMgLevel), P(OrcOp), C.c_int, _dp, _dp]
        L.orc_topo_u1.argtypes = [_dp, C.c_int, C.c_int]
        L.orc_topo_u1.restype = C.c_double
        L.orc_gauge_trans_u1.argtypes = [_dp, _dp, C.c_int, C.c_int]
        L.orc_ape_smear_u1.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int]
        L.orc_eoprec_reconstruct.argtypes = [P(OrcOp), _dp, _dp, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int

    def set_threads(self, n=None):
        """Threads for the oracle's site loops (operators and vector updates); reductions stay
        serial in the reference's order, so results do not depend on n.  None: every core."""
        self.lib.orc_set_threads(int(n) if n else (os.cpu_count() or 1))
        return self.lib.orc_get_threads()

    def apply(self, op: Operator, rhs):
        rhs = np.ascontiguousarray(rhs, dtype=np.complex128)
        lhs = np.empty_like(rhs)
        self.lib.orc_apply(C.byref(op.struct), _ptr(lhs), _ptr(rhs))
        return lhs

    def eoprec_prepare(self, op: Operator, rhs):
        rhs = np.ascontiguousarray(rhs, dtype=np.complex128)
        out = np.empty_like(rhs)
        self.lib.orc_eoprec_prepare(C.byref(op.struct), _ptr(out), _ptr(rhs))
        return out

    def eoprec_reconstruct(self, op: Operator, lhs_e, rhs_o):
        lhs_e = np.ascontiguousarray(lhs_e, dtype=np.complex128)
        rhs_o = np.ascontiguousarray(rhs_o, dtype=np.complex128)
        out = np.empty_like(lhs_e)
        self.lib.orc_eoprec_reconstruct(C.byref(op.struct), _ptr(out), _ptr(lhs_e), _ptr(rhs_o))
        return out

    def staggered_stencil(self, links, lx, ly, dagger=False):
        links = np.ascontiguousarray(links, dtype=np.complex128)
        hop = np.zeros(4 * lx * ly, dtype=np.complex128)
        self.lib.orc_staggered_stencil(_ptr(hop), _ptr(links), lx, ly, int(dagger))
        return hop

    def dot(self, a, b):
        out = np.zeros(2)
        self.lib.orc_dot(_ptr(a), _ptr(b), a.size, _ptr(out))
        return complex(out[0], out[1])

    def norm2sq(self, a):
        return self.lib.orc_norm2sq(_ptr(a), a.size)

    def solve(self, solver, op: Operator, phi0, phi=None, max_iter=10000, eps=1e-10,
              restart_freq=0, hist_cap=0):
        """solver in {"cg", "bicgstab", "gcr"}; returns (phi, info dict, hist)."""
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        phi = np.zeros_like(phi0) if phi is None else np.array(phi, dtype=np.complex128)
        info = OrcInfo()
        hist = np.zeros(max(hist_cap, 1))
        if restart_freq > 0:
            getattr(self.lib, f"orc_{solver}_restart")(C.byref(op.struct), _ptr(phi), _ptr(phi0),
                                                       phi0.size, max_iter, eps, restart_freq,
                                                       C.byref(info))
        else:
            getattr(self.lib, f"orc_{solver}")(C.byref(op.struct), _ptr(phi), _ptr(phi0), phi0.size,
                                               max_iter, eps, C.byref(info),
                                               _ptr(hist) if hist_cap else None, hist_cap)
        d = info.as_dict()
        return phi, d, hist[: min(hist_cap, d["iter"])] if hist_cap else None

    def cg_m(self, op: Operator, phi0, shifts, resid_freq_check=1, max_iter=10000, eps=1e-10,
             worst_first=False, hist_cap=0):
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        shifts = np.ascontiguousarray(shifts, dtype=np.float64)
        ns = shifts.size
        phi = np.zeros((ns, phi0.size), dtype=np.complex128)
        res = np.zeros(ns)
        hist = np.zeros(max(hist_cap, 1))
        info = OrcInfo()
        self.lib.orc_cg_m(C.byref(op.struct), _ptr(phi), _ptr(phi0), ns, phi0.size,
                          resid_freq_check, max_iter, eps, _ptr(shifts), int(worst_first),
                          C.byref(info), _ptr(res), _ptr(hist) if hist_cap else None, hist_cap)
        return phi, info.as_dict(), res

    def solve2(self, solver, op: Operator, phi0, phi=None, max_iter=10000, eps=1e-10,
               restart_freq=0, l=2, omega=1.0, precond="identity", n_step=4, rel_res=1e-1,
               hist_cap=0):
        """The sibling solvers: solver in {"cr", "minres", "bicgstab_l", "fpcg", "vpgcr"};
        the preconditioner of fpcg / vpgcr runs on op itself.  Returns (phi, info, hist)."""
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        phi = np.zeros_like(phi0) if phi is None else np.array(phi, dtype=np.complex128)
        info = OrcInfo()
        hist = np.zeros(max(hist_cap, 1))
        hp = _ptr(hist) if hist_cap else None
        a = (C.byref(op.struct), _ptr(phi), _ptr(phi0), phi0.size, max_iter, eps)
        pc = OrcPrecond(PRECOND[precond], n_step, rel_res, C.pointer(op.struct))
        L = self.lib
        if solver == "cr":
            if restart_freq > 0: L.orc_cr_restart(*a, restart_freq, C.byref(info))
            else: L.orc_cr(*a, C.byref(info), hp, hist_cap)
        elif solver == "minres":
            L.orc_minres(*a, omega, C.byref(info), hp, hist_cap)
        elif solver == "bicgstab_l":
            if restart_freq > 0: L.orc_bicgstab_l_restart(*a, restart_freq, l, C.byref(info))
            else: L.orc_bicgstab_l(*a, l, C.byref(info), hp, hist_cap)
        else:
            if restart_freq > 0: getattr(L, f"orc_{solver}_restart")(*a, restart_freq, C.byref(pc), C.byref(info))
            else: getattr(L, f"orc_{solver}")(*a, C.byref(pc), C.byref(info), hp, hist_cap)
        d = info.as_dict()
        return phi, d, hist[: min(hist_cap, max(d["iter"], 0))] if hist_cap else None

    def multishift(self, solver, op: Operator, phi0, shifts, resid_freq_check=1, max_iter=10000,
                   eps=1e-10, worst_first=False, hist_cap=0):
        """solver in {"cg_m", "cr_m", "bicgstab_m"}."""
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        shifts = np.ascontiguousarray(shifts, dtype=np.float64)
        ns = shifts.size
        phi = np.zeros((ns, phi0.size), dtype=np.complex128)
        res = np.zeros(ns)
        hist = np.zeros(max(hist_cap, 1))
        info = OrcInfo()
        getattr(self.lib, f"orc_{solver}")(C.byref(op.struct), _ptr(phi), _ptr(phi0), ns, phi0.size,
                                           resid_freq_check, max_iter, eps, _ptr(shifts), int(worst_first),
                                           C.byref(info), _ptr(res), _ptr(hist) if hist_cap else None,
                                           hist_cap)
        return phi, info.as_dict(), res

    def tbprec_prepare(self, op: Operator, rhs):
        rhs = np.ascontiguousarray(rhs, dtype=np.complex128)
        out = np.empty_like(rhs)
        self.lib.orc_tbprec_prepare(C.byref(op.struct), _ptr(out), _ptr(rhs))
        return out

    def tbprec_reconstruct(self, op: Operator, lhs_t, rhs_b):
        lhs_t = np.ascontiguousarray(lhs_t, dtype=np.complex128)
        rhs_b = np.ascontiguousarray(rhs_b, dtype=np.complex128)
        out = np.empty_like(lhs_t)
        self.lib.orc_tbprec_reconstruct(C.byref(op.struct), _ptr(out), _ptr(lhs_t), _ptr(rhs_b))
        return out

    @staticmethod
    def _mg(lx, ly, nc_f, bx, by, nc_c, nv):
        return OrcMgLevel(lx, ly, nc_f, bx, by, nc_c, _ptr(nv))

    def mg_block(self, which, lx, ly, nc_f, bx, by, nc_c, null_vectors):
        """which: "normalize" or "orthonormalize"; returns the new vectors (nc_c, lx*ly*nc_f)."""
        nv = np.array(null_vectors, dtype=np.complex128).reshape(nc_c, -1).copy()
        lv = self._mg(lx, ly, nc_f, bx, by, nc_c, nv)
        getattr(self.lib, f"orc_mg_block_{which}")(C.byref(lv))
        return nv

    def mg_prolong(self, lx, ly, nc_f, bx, by, nc_c, null_vectors, coarse):
        nv = np.ascontiguousarray(null_vectors, dtype=np.complex128)
        out = np.zeros(lx * ly * nc_f, np.complex128)
        self.lib.orc_mg_prolong(C.byref(self._mg(lx, ly, nc_f, bx, by, nc_c, nv)), _ptr(out),
                                _ptr(np.ascontiguousarray(coarse, dtype=np.complex128)))
        return out

    def mg_restrict(self, lx, ly, nc_f, bx, by, nc_c, null_vectors, fine):
        nv = np.ascontiguousarray(null_vectors, dtype=np.complex128)
        out = np.zeros((lx // bx) * (ly // by) * nc_c, np.complex128)
        self.lib.orc_mg_restrict(C.byref(self._mg(lx, ly, nc_f, bx, by, nc_c, nv)), _ptr(out),
                                 _ptr(np.ascontiguousarray(fine, dtype=np.complex128)))
        return out

    def mg_coarse_stencil(self, lx, ly, nc_f, bx, by, nc_c, null_vectors, fine: Operator, ignore_shifts=False):
        nv = np.ascontiguousarray(null_vectors, dtype=np.complex128)
        vc = (lx // bx) * (ly // by) * nc_c * nc_c
        clov, hop = np.zeros(vc, np.complex128), np.zeros(4 * vc, np.complex128)
        self.lib.orc_mg_coarse_stencil(C.byref(self._mg(lx, ly, nc_f, bx, by, nc_c, nv)), C.byref(fine.struct),
                                       int(ignore_shifts), _ptr(clov), _ptr(hop))
        return clov, hop

    def plaquette(self, links, lx, ly):
        out = np.zeros(2)
        self.lib.orc_plaquette_u1(_ptr(np.ascontiguousarray(links)), lx, ly, _ptr(out))
        return complex(out[0], out[1])

    def topo(self, links, lx, ly):
        return self.lib.orc_topo_u1(_ptr(np.ascontiguousarray(links)), lx, ly)

    def gauge_trans(self, links, trans, lx, ly):
        out = np.array(links, dtype=np.complex128)
        self.lib.orc_gauge_trans_u1(_ptr(out), _ptr(np.ascontiguousarray(trans)), lx, ly)
        return out

    def ape_smear(self, links, lx, ly, alpha, n_iter):
        out = np.zeros(2 * lx * ly, np.complex128)
        self.lib.orc_ape_smear_u1(_ptr(out), _ptr(np.ascontiguousarray(links)), lx, ly, alpha, n_iter)
        return out

    def staggered_force(self, links, mass, lx, ly, X, Y):
        out = np.zeros(2 * lx * ly)
        self.lib.orc_staggered_force(_ptr(np.ascontiguousarray(links)), mass, lx, ly,
                                     _ptr(np.ascontiguousarray(X)), _ptr(np.ascontiguousarray(Y)),
                                     _ptr(out))
        return out


class RefOracle:
    """The reference's own code (compiled from its sources); available only where the
    reference checkout exists."""

    def __init__(self, path=REF_LIB_PATH):
        L = C.CDLL(path)
        self.lib = L
        cp = C.c_char_p
        L.ref_make_inputs.argtypes = [C.c_uint, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_long]
        L.ref_gauss_gauge.argtypes = [C.c_uint, C.c_int, C.c_int, C.c_double, _dp]
        L.ref_read_gauge.argtypes = [cp, C.c_int, C.c_int, _dp]
        opargs = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp]
        L.ref_apply.argtypes = opargs + [_dp, _dp]
        L.ref_staggered_stencil.argtypes = [C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp, _dp]
        L.ref_solve.argtypes = [C.c_int, C.c_int] + opargs + [_dp, _dp, C.c_int, C.c_double, C.c_int,
                                                              cp, _dp, C.c_char_p, C.c_int, C.c_char_p, C.c_int]
        L.ref_cg_m.argtypes = opargs + [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int,
                                        C.c_int, cp, _dp, _dp, C.c_char_p, C.c_int]
        L.ref_solve2.argtypes = [C.c_int, C.c_int] + opargs + [_dp, _dp, C.c_int, C.c_double, C.c_int,
                                                               C.c_double, C.c_int, C.c_int, C.c_double,
                                                               C.c_int, cp, C.c_int, cp, _dp, C.c_char_p,
                                                               C.c_int, C.c_char_p, C.c_int]
        L.ref_multishift2.argtypes = [C.c_int] + L.ref_cg_m.argtypes
        L.ref_eoprec_prepare.argtypes = opargs + [_dp, _dp]
        L.ref_plaquette.argtypes = [_dp, C.c_int, C.c_int, _dp]
        L.ref_tbprec.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_mg_block.argtypes = [C.c_int] + [C.c_int] * 6 + [_dp]
        L.ref_mg_transfer.argtypes = [C.c_int] + [C.c_int] * 6 + [_dp, _dp, _dp]
        L.ref_mg_coarse.argtypes = [C.c_int] * 6 + [_dp, _dp, _dp, _dp, C.c_int, _dp, _dp]
        ip = C.POINTER(C.c_int)
        L.ref_mg_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int, ip, ip, _dp, C.c_int, ip,
                                   ip, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp, C.c_int, C.c_double, _dp,
                                   C.c_char_p, C.c_int]
        L.ref_topo.argtypes = [_dp, C.c_int, C.c_int]
        L.ref_topo.restype = C.c_double
        L.ref_gauge_trans.argtypes = [C.c_uint, _dp, _dp, C.c_int, C.c_int]
        L.ref_ape_smear.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_int]
        L.ref_write_gauge.argtypes = [cp, _dp, C.c_int, C.c_int]
        L.ref_unit_gauge.argtypes = [_dp, C.c_int, C.c_int]
        L.ref_eoprec_reconstruct.argtypes = opargs + [_dp, _dp, _dp]

    def make_inputs(self, seed, lx, ly, n_src=1, src_len=None):
        links = np.zeros(2 * lx * ly, dtype=np.complex128)
        src_len = lx * ly if src_len is None else src_len
        src = np.zeros((n_src, src_len), dtype=np.complex128)
        self.lib.ref_make_inputs(seed, lx, ly, _ptr(links), _ptr(src), n_src, src_len)
        return links, src

    def read_gauge(self, path, lx, ly):
        links = np.zeros(2 * lx * ly, dtype=np.complex128)
        self.lib.ref_read_gauge(path.encode(), lx, ly, _ptr(links))
        return links

    def _opargs(self, op: Operator):
        return (op.kind, op.lx, op.ly, op.nc, op.mass, _ptr(op.links), _ptr(op.clover),
                _ptr(op.hopping), _ptr(op.two_link), _ptr(op._s6))

    def apply(self, op: Operator, rhs):
        op._s6 = op.shifts6()
        rhs = np.ascontiguousarray(rhs, dtype=np.complex128)
        lhs = np.zeros_like(rhs)
        self.lib.ref_apply(*self._opargs(op), _ptr(lhs), _ptr(rhs))
        return lhs

    def eoprec_prepare(self, op: Operator, rhs):
        op._s6 = op.shifts6()
        rhs = np.ascontiguousarray(rhs, dtype=np.complex128)
        out = np.zeros_like(rhs)
        self.lib.ref_eoprec_prepare(*self._opargs(op), _ptr(out), _ptr(rhs))
        return out

    def eoprec_reconstruct(self, op: Operator, lhs_e, rhs_o):
        op._s6 = op.shifts6()
        lhs_e = np.ascontiguousarray(lhs_e, dtype=np.complex128)
        rhs_o = np.ascontiguousarray(rhs_o, dtype=np.complex128)
        out = np.zeros_like(lhs_e)
        self.lib.ref_eoprec_reconstruct(*self._opargs(op), _ptr(out), _ptr(lhs_e), _ptr(rhs_o))
        return out

    def staggered_stencil(self, links, lx, ly, mass, dagger=False):
        hop = np.zeros(4 * lx * ly, dtype=np.complex128)
        sh = np.zeros(2)
        self.lib.ref_staggered_stencil(lx, ly, mass, _ptr(np.ascontiguousarray(links)), int(dagger),
                                       _ptr(hop), _ptr(sh))
        return hop, complex(sh[0], sh[1])

    def solve(self, solver, op: Operator, phi0, phi=None, max_iter=10000, eps=1e-10,
              restart_freq=0, verbosity=0, prefix=""):
        op._s6 = op.shifts6()
        sid = {"cg": 0, "bicgstab": 1, "gcr": 2}[solver]
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        phi = np.zeros_like(phi0) if phi is None else np.array(phi, dtype=np.complex128)
        info = np.zeros(4)
        name = C.create_string_buffer(64)
        log = C.create_string_buffer(1 << 20)
        self.lib.ref_solve(sid, restart_freq, *self._opargs(op), _ptr(phi), _ptr(phi0), max_iter, eps,
                           verbosity, prefix.encode(), _ptr(info), name, 64, log, 1 << 20)
        d = {"resSq": info[0], "iter": int(info[1]), "success": bool(info[2]),
             "ops_count": int(info[3]), "name": name.value.decode()}
        return phi, d, log.value.decode()

    def cg_m(self, op: Operator, phi0, shifts, resid_freq_check=1, max_iter=10000, eps=1e-10,
             worst_first=False, verbosity=0, prefix=""):
        op._s6 = op.shifts6()
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        shifts = np.array(shifts, dtype=np.float64)
        ns = shifts.size
        phi = np.zeros((ns, phi0.size), dtype=np.complex128)
        info = np.zeros(4)
        res = np.zeros(ns)
        log = C.create_string_buffer(1 << 20)
        self.lib.ref_cg_m(*self._opargs(op), _ptr(phi), _ptr(phi0), ns, resid_freq_check, max_iter,
                          eps, _ptr(shifts), int(worst_first), verbosity, prefix.encode(), _ptr(info),
                          _ptr(res), log, 1 << 20)
        d = {"resSq": info[0], "iter": int(info[1]), "success": bool(info[2]),
             "ops_count": int(info[3]), "name": "CG-M"}
        return phi, d, res, log.value.decode()

    def solve2(self, solver, op: Operator, phi0, phi=None, max_iter=10000, eps=1e-10,
               restart_freq=0, l=2, omega=1.0, precond="identity", n_step=4, rel_res=1e-1,
               verbosity=0, prefix="", precond_verbosity=0, precond_prefix=""):
        """The reference's sibling solvers (see Oracle.solve2); returns (phi, info, log)."""
        op._s6 = op.shifts6()
        sid = {"cr": 3, "minres": 4, "bicgstab_l": 5, "fpcg": 6, "vpgcr": 7}[solver]
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        phi = np.zeros_like(phi0) if phi is None else np.array(phi, dtype=np.complex128)
        info = np.zeros(4)
        name = C.create_string_buffer(64)
        log = C.create_string_buffer(1 << 21)
        self.lib.ref_solve2(sid, restart_freq, *self._opargs(op), _ptr(phi), _ptr(phi0), max_iter, eps,
                            l, omega, PRECOND[precond], n_step, rel_res, verbosity, prefix.encode(),
                            precond_verbosity, precond_prefix.encode(), _ptr(info), name, 64, log, 1 << 21)
        d = {"resSq": info[0], "iter": int(info[1]), "success": bool(info[2]),
             "ops_count": int(info[3]), "name": name.value.decode()}
        return phi, d, log.value.decode()

    def multishift(self, solver, op: Operator, phi0, shifts, resid_freq_check=1, max_iter=10000,
                   eps=1e-10, worst_first=False, verbosity=0, prefix=""):
        """solver in {"cr_m", "bicgstab_m"}; returns (phi, info, resSqmrhs, log)."""
        op._s6 = op.shifts6()
        phi0 = np.ascontiguousarray(phi0, dtype=np.complex128)
        shifts = np.array(shifts, dtype=np.float64)
        ns = shifts.size
        phi = np.zeros((ns, phi0.size), dtype=np.complex128)
        info = np.zeros(4)
        res = np.zeros(ns)
        log = C.create_string_buffer(1 << 20)
        self.lib.ref_multishift2({"cr_m": 0, "bicgstab_m": 1}[solver], *self._opargs(op), _ptr(phi),
                                 _ptr(phi0), ns, resid_freq_check, max_iter, eps, _ptr(shifts),
                                 int(worst_first), verbosity, prefix.encode(), _ptr(info), _ptr(res),
                                 log, 1 << 20)
        d = {"resSq": info[0], "iter": int(info[1]), "success": bool(info[2]),
             "ops_count": int(info[3]), "name": {"cr_m": "CR-M", "bicgstab_m": "BICGSTAB-M"}[solver]}
        return phi, d, res, log.value.decode()

    def plaquette(self, links, lx, ly):
        out = np.zeros(2)
        self.lib.ref_plaquette(_ptr(np.ascontiguousarray(links)), lx, ly, _ptr(out))
        return complex(out[0], out[1])

    def topo(self, links, lx, ly):
        return self.lib.ref_topo(_ptr(np.ascontiguousarray(links)), lx, ly)

    def gauge_trans(self, seed, links, lx, ly):
        """rand_trans_u1 from std::mt19937(seed), then apply_gauge_trans_u1; (links', trans)."""
        out = np.array(links, dtype=np.complex128)
        trans = np.zeros(lx * ly, np.complex128)
        self.lib.ref_gauge_trans(seed, _ptr(out), _ptr(trans), lx, ly)
        return out, trans

    def ape_smear(self, links, lx, ly, alpha, n_iter):
        out = np.zeros(2 * lx * ly, np.complex128)
        self.lib.ref_ape_smear(_ptr(out), _ptr(np.ascontiguousarray(links)), lx, ly, alpha, n_iter)
        return out

    def write_gauge(self, path, links, lx, ly):
        self.lib.ref_write_gauge(path.encode(), _ptr(np.ascontiguousarray(links)), lx, ly)

    def tbprec(self, step, op: Operator, a, b=None):
        """step 0: tbprec prepare (a = rhs); step 1: reconstruct (a = lhs_t, b = rhs_b)."""
        a = np.ascontiguousarray(a, dtype=np.complex128)
        out = np.zeros_like(a)
        self.lib.ref_tbprec(step, op.lx, op.ly, op.nc, _ptr(op.clover), _ptr(op.hopping), _ptr(op.shifts6()),
                            _ptr(out), _ptr(a), _ptr(None if b is None else np.ascontiguousarray(b)))
        return out

    def mg_block(self, which, lx, ly, nc_f, bx, by, nc_c, null_vectors):
        nv = np.array(null_vectors, dtype=np.complex128).reshape(nc_c, -1).copy()
        self.lib.ref_mg_block({"normalize": 0, "orthonormalize": 1}[which], lx, ly, nc_f, bx, by, nc_c, _ptr(nv))
        return nv

    def mg_prolong(self, lx, ly, nc_f, bx, by, nc_c, null_vectors, coarse):
        nv = np.array(null_vectors, dtype=np.complex128)
        out = np.zeros(lx * ly * nc_f, np.complex128)
        self.lib.ref_mg_transfer(0, lx, ly, nc_f, bx, by, nc_c, _ptr(nv), _ptr(out),
                                 _ptr(np.ascontiguousarray(coarse, dtype=np.complex128)))
        return out

    def mg_restrict(self, lx, ly, nc_f, bx, by, nc_c, null_vectors, fine):
        nv = np.array(null_vectors, dtype=np.complex128)
        out = np.zeros((lx // bx) * (ly // by) * nc_c, np.complex128)
        self.lib.ref_mg_transfer(1, lx, ly, nc_f, bx, by, nc_c, _ptr(nv), _ptr(out),
                                 _ptr(np.ascontiguousarray(fine, dtype=np.complex128)))
        return out

    def mg_coarse_stencil(self, lx, ly, nc_f, bx, by, nc_c, null_vectors, fine: Operator, ignore_shifts=False):
        nv = np.array(null_vectors, dtype=np.complex128)
        vc = (lx // bx) * (ly // by) * nc_c * nc_c
        clov, hop = np.zeros(vc, np.complex128), np.zeros(4 * vc, np.complex128)
        self.lib.ref_mg_coarse(lx, ly, nc_f, bx, by, nc_c, _ptr(nv), _ptr(fine.clover), _ptr(fine.hopping),
                               _ptr(fine.shifts6()), int(ignore_shifts), _ptr(clov), _ptr(hop))
        return clov, hop

    def mg_solve(self, outer, links, lx, ly, mass, b, blocks, nvecs, null_vectors, smoother, n_pre, n_post,
                 inner, n_max, n_restart, rel_res, mlevel=0, max_iter=10000, eps=1e-10):
        """The reference's flexible solve (outer "fpcg" / "vpgcr") preconditioned by its
        mg_preconditioner; null_vectors: the concatenated Gaussian inputs of every level.
        Returns (phi, info, log)."""
        nr = len(blocks)
        I = lambda a: (C.c_int * len(a))(*a)
        nv = np.array(null_vectors, dtype=np.complex128).reshape(-1).copy()
        phi = np.zeros(lx * ly, np.complex128)
        b = np.ascontiguousarray(b, dtype=np.complex128)
        info = np.zeros(4)
        log = C.create_string_buffer(1 << 22)
        rr = np.ascontiguousarray(rel_res, dtype=np.float64)
        self.lib.ref_mg_solve({"fpcg": 0, "vpgcr": 1}[outer], lx, ly, mass, _ptr(np.ascontiguousarray(links)), nr,
                              I(blocks), I(nvecs), _ptr(nv), smoother, I(n_pre), I(n_post), inner, n_max, n_restart,
                              _ptr(rr), mlevel, _ptr(phi), _ptr(b), max_iter, eps, _ptr(info), log, 1 << 22)
        d = {"resSq": info[0], "iter": int(info[1]), "success": bool(info[2]), "ops_count": int(info[3])}
        return phi, d, log.value.decode()
