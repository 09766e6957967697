"""The CPU oracle's sibling Krylov solvers against the reference's own outputs (golden
fixtures from generic_cr.cpp, generic_minres.cpp, generic_bicgstab_l.cpp,
generic_cr_m.cpp, generic_bicgstab_m.cpp, generic_cg_flex_precond.cpp and
generic_gcr_var_precond.cpp compiled from the reference's sources).  Bit-exact: the oracle
keeps the reference's operation order, its iteration and operator counts, its stopping rules
(including the complex CR's success test against k == max_iter, generic_cr.cpp:288, which makes
the restarted CR stop after one cycle) and its verbosity output."""
from __future__ import annotations

import numpy as np
import pytest

from pyoracle import Operator

MASS = {"staggered_normal": 0.1, "staggered": 0.1, "laplace_m0.5": 0.5, "laplace_m0.001": 0.001}


def _op(name, links):
    kind = name.split("_m0")[0]
    return Operator(kind, 32, 32, MASS[name], links)


def _sib_keys(cases):
    return sorted(k for k, c in cases.items() if "solver" in c and "maxiter" not in k)


def pytest_generate_tests(metafunc):
    if "sib_key" in metafunc.fixturenames:
        import json, os
        here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_info.json")
        cases = json.load(open(here))["cases"]
        metafunc.parametrize("sib_key", _sib_keys(cases))


def test_sibling_solvers_bit_exact(oracle, golden, sib_key):
    vec, cases = golden
    c = cases[sib_key]
    x, info, _ = oracle.solve2(c["solver"], _op(c["op"], vec["l32_links"]), vec["l32_src"],
                               max_iter=c["max_iter"], eps=c["eps"], **c["kw"])
    for f in ("iter", "ops_count", "success", "name"):
        assert info[f] == c[f], f
    assert info["resSq"] == c["resSq"]
    assert np.array_equal(x, vec[sib_key])


@pytest.mark.parametrize("key", ["l32_cr_maxiter6", "l32_minres_maxiter5", "l32_bicgstab_l_maxiter6",
                                 "l32_fpcg_maxiter4", "l32_vpgcr_maxiter4"])
def test_sibling_max_iter_paths(oracle, golden, key):
    """Cut at max_iter: the reference's counts and success flag, and the relative residuals
    its DETAIL log prints (one line per iteration; per l-cycle for BiCGstab-l)."""
    vec, cases = golden
    c = cases[key]
    _, info, hist = oracle.solve2(c["solver"], _op(c["op"], vec["l32_links"]), vec["l32_src"],
                                  max_iter=c["max_iter"], hist_cap=c["max_iter"], **c["kw"])
    assert (info["iter"], info["ops_count"], info["success"]) == (c["iter"], c["ops_count"], c["success"])
    assert info["resSq"] == c["resSq"]
    logged = [float(l.split("RelRes ")[1]) for l in c["log"].splitlines() if " Iter " in l and "Success" not in l]
    assert len(logged) >= 1
    assert np.allclose(hist[: len(logged)], logged, rtol=1e-5)


@pytest.mark.parametrize("solver", ["cr_m", "bicgstab_m"])
@pytest.mark.parametrize("rfc,wf", [(1, 0), (3, 0), (1, 1)])
def test_multishift_siblings_bit_exact(oracle, golden, solver, rfc, wf):
    vec, cases = golden
    key = f"l32_{solver}_rfc{rfc}_wf{wf}"
    c = cases[key]
    x, info, res = oracle.multishift(solver, _op(c["op"], vec["l32_links"]), vec["l32_src"], c["shifts"],
                                     resid_freq_check=rfc, worst_first=bool(wf))
    assert (info["iter"], info["ops_count"], info["success"], info["name"]) == \
        (c["iter"], c["ops_count"], c["success"], c["name"])
    assert np.array_equal(res, np.array(c["resSqmrhs"]))
    assert np.array_equal(x.reshape(-1), vec[key])


def test_multishift_solutions_solve_shifted_systems(golden):
    """Each CR-M / BiCGstab-M solution solves (A + sigma) x = b (the reference's own
    explicit residuals, resSqmrhs, are below (1e-10 |b|)^2 up to the recurrences' drift)."""
    vec, cases = golden
    bsq = float(np.vdot(vec["l32_src"], vec["l32_src"]).real)
    for solver in ("cr_m", "bicgstab_m"):
        c = cases[f"l32_{solver}_rfc1_wf0"]
        assert max(c["resSqmrhs"]) < (1e-9) ** 2 * bsq
