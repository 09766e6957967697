"""Writes the golden fixtures in this directory from the reference's own code.

The reference's operators, stencil builders, solvers and input generators are compiled from
the reference checkout (``make -C oracle ref``, sources read in place) into
oracle/_ref/libref_oracle.so; this script calls them through ctypes on seeded inputs and
stores inputs, outputs, solver infos and verbosity logs:

  reference_vectors.npz   complex128 fields (inputs and outputs)
  reference_info.json     solver infos, verbosity logs, parameters

Run from the repository root:
  GLINALG_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
(or without the variable after a build that compiled the reference and recorded its location).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402


def main():
    refdir = pyoracle.reference_dir()
    if not refdir:
        raise SystemExit("set GLINALG_REFERENCE_DIR to the reference checkout")
    pyoracle.build(reference=refdir)
    R = pyoracle.RefOracle()
    Op = pyoracle.Operator
    vec = {}
    info = {"cases": {}}

    # ---- inputs: std::mt19937(seed) -> rand_gauge_u1 -> gaussian source(s)
    lat = {"l32": (32, 32, 1337), "l8": (8, 8, 7), "l12x6": (12, 6, 3)}
    for key, (lx, ly, seed) in lat.items():
        links, src = R.make_inputs(seed, lx, ly, 2)
        vec[f"{key}_links"], vec[f"{key}_src"], vec[f"{key}_src2"] = links, src[0], src[1]
        info["cases"][key] = {"lx": lx, "ly": ly, "seed": seed}
    # gauss_gauge_u1 with beta = 6 (a smooth field), seed 11, 16x16
    vec["g16_links"] = np.zeros(2 * 256, np.complex128)
    R.lib.ref_gauss_gauge(11, 16, 16, 6.0, vec["g16_links"].ctypes.data_as(pyoracle._dp))
    info["cases"]["g16"] = {"lx": 16, "ly": 16, "seed": 11, "beta": 6.0}

    # ---- operators (operators.cpp)
    for key in ("l32", "l8", "l12x6"):
        lx, ly, _ = lat[key]
        U, b = vec[f"{key}_links"], vec[f"{key}_src"]
        for kind in ("staggered", "staggered_dagger", "staggered_normal"):
            vec[f"{key}_{kind}"] = R.apply(Op(kind, lx, ly, 0.1, U), b)
        vec[f"{key}_laplace"] = R.apply(Op("laplace", lx, ly, 0.01, U), b)
        # stencil builders (operators_stencil.cpp) and the stencil applied to the source
        for dag in (0, 1):
            hop, sh = R.staggered_stencil(U, lx, ly, 0.1, bool(dag))
            vec[f"{key}_stencil_hop{dag}"] = hop
            vec[f"{key}_stencil_apply{dag}"] = R.apply(
                Op("stencil", lx, ly, nc=1, clover=np.zeros(lx * ly, np.complex128), hopping=hop, shift=sh), b)

    # ---- generic stencil, Nc = 3, with and without two-link terms, all three parities
    rng = np.random.default_rng(2024)
    lx, ly, nc = 6, 4, 3
    v = lx * ly * nc * nc
    cl = rng.normal(size=v) + 1j * rng.normal(size=v)
    hp = rng.normal(size=4 * v) + 1j * rng.normal(size=4 * v)
    tl = rng.normal(size=8 * v) + 1j * rng.normal(size=8 * v)
    x = rng.normal(size=lx * ly * nc) + 1j * rng.normal(size=lx * ly * nc)
    vec.update({"st3_clover": cl, "st3_hopping": hp, "st3_two": tl, "st3_x": x})
    shifts = {"shift": 0.3 + 0.1j, "eo_shift": 0.2 - 0.05j, "dof_shift": -0.4j}
    info["cases"]["st3"] = {"lx": lx, "ly": ly, "nc": nc, **{k: [z.real, z.imag] for k, z in shifts.items()}}
    for kind in ("stencil", "stencil_eo", "stencil_oe"):
        for two in (0, 1):
            o = Op(kind, lx, ly, nc=nc, clover=cl, hopping=hp, two_link=tl if two else None, **shifts)
            vec[f"st3_{kind}_two{two}"] = R.apply(o, x)

    # ---- solvers on the 32x32 system (m = 0.1, tol 1e-10)
    lx, ly = 32, 32
    U, b = vec["l32_links"], vec["l32_src"]
    normal = Op("staggered_normal", lx, ly, 0.1, U)
    stag = Op("staggered", lx, ly, 0.1, U)
    solves = [
        ("cg", normal, 0), ("cg", normal, 17), ("bicgstab", stag, 0), ("bicgstab", stag, 17),
        ("gcr", stag, 0), ("gcr", stag, 17),
    ]
    for solver, op, rf in solves:
        x0 = np.zeros_like(b)
        xs, d, log = R.solve(solver, op, b, phi=x0, max_iter=10000, eps=1e-10, restart_freq=rf,
                             verbosity=1 if rf == 0 else 2, prefix="[GOLD] ")
        key = f"l32_{solver}" + (f"_r{rf}" if rf else "")
        vec[key] = xs
        info["cases"][key] = {**{k: (bool(v_) if isinstance(v_, (bool, np.bool_)) else v_) for k, v_ in d.items()},
                              "log": log, "restart_freq": rf, "max_iter": 10000, "eps": 1e-10,
                              "op": "staggered_normal" if op is normal else "staggered"}
    # detail-level log and a max_iter cut for CG (success == false path)
    _, d, log = R.solve("cg", normal, b, max_iter=7, eps=1e-10, verbosity=3, prefix="[CG] ")
    info["cases"]["l32_cg_maxiter7"] = {**d, "log": log}
    _, d, log = R.solve("bicgstab", stag, b, max_iter=5, eps=1e-10, verbosity=3, prefix="")
    info["cases"]["l32_bicgstab_maxiter5"] = {**d, "log": log}
    _, d, log = R.solve("gcr", stag, b, max_iter=5, eps=1e-10, verbosity=3, prefix="")
    info["cases"]["l32_gcr_maxiter5"] = {**d, "log": log}
    # initial guess honoured: CG started from src2
    xs, d, _ = R.solve("cg", normal, b, phi=vec["l32_src2"], max_iter=10000, eps=1e-10)
    vec["l32_cg_guess"] = xs
    info["cases"]["l32_cg_guess"] = d

    # ---- multishift CG on the gauge Laplacian (tests/multishift/multishift.cpp:424-494 style)
    lap = Op("laplace", lx, ly, 0.001, U)
    msh = [0.0, 0.004, 0.009, 0.049, 0.099, 0.499, 0.999]
    for rfc, wf in ((1, False), (3, False), (1, True)):
        xs, d, res, log = R.cg_m(lap, b, msh, resid_freq_check=rfc, max_iter=10000, eps=1e-10,
                                 worst_first=wf, verbosity=1, prefix="[CGM] ")
        key = f"l32_cgm_rfc{rfc}_wf{int(wf)}"
        vec[key] = xs.reshape(-1)
        info["cases"][key] = {**d, "resSqmrhs": res.tolist(), "log": log, "shifts": msh,
                              "rfc": rfc, "worst_first": wf, "mass": 0.001}

    # ---- even/odd preconditioning (operators.cpp:455-620, operators_stencil.cpp:179-236)
    for key in ("l32", "l8", "l12x6"):
        lx, ly, _ = lat[key]
        U, b_, b2 = vec[f"{key}_links"], vec[f"{key}_src"], vec[f"{key}_src2"]
        for kind in ("staggered_deo", "staggered_doe", "staggered_m2mdeodoe"):
            vec[f"{key}_{kind}"] = R.apply(Op(kind, lx, ly, 0.1, U), b_)
        eo = Op("staggered_m2mdeodoe", lx, ly, 0.1, U)
        vec[f"{key}_eo_prepare"] = R.eoprec_prepare(eo, b_)
        vec[f"{key}_eo_reconstruct"] = R.eoprec_reconstruct(eo, b2, b_)
    # the stencil form on the 8x8 staggered stencil (shift = mass)
    lx, ly = 8, 8
    hop, sh = R.staggered_stencil(vec["l8_links"], lx, ly, 0.1, False)
    seo = Op("stencil_m2mdeodoe", lx, ly, nc=1, clover=np.zeros(lx * ly, np.complex128), hopping=hop, shift=sh)
    vec["l8_stencil_m2mdeodoe"] = R.apply(seo, vec["l8_src"])
    vec["l8_stencil_eo_prepare"] = R.eoprec_prepare(seo, vec["l8_src"])
    vec["l8_stencil_eo_reconstruct"] = R.eoprec_reconstruct(seo, vec["l8_src2"], vec["l8_src"])
    # M x = b on the 32x32 system by even/odd preconditioning (tests/staggered_pieces/
    # staggered_pieces.cpp:331-346): prepare, CG on m^2 - D_eo D_oe, reconstruct
    lx, ly = 32, 32
    U, b_ = vec["l32_links"], vec["l32_src"]
    eo = Op("staggered_m2mdeodoe", lx, ly, 0.1, U)
    rhs_e = R.eoprec_prepare(eo, b_)
    xe, d, log = R.solve("cg", eo, rhs_e, max_iter=10000, eps=1e-10, verbosity=1, prefix="[EO] ")
    vec["l32_eo_cg_even"] = xe
    vec["l32_eo_solution"] = R.eoprec_reconstruct(eo, xe, b_)
    info["cases"]["l32_eo_cg"] = {**d, "log": log, "max_iter": 10000, "eps": 1e-10, "mass": 0.1}

    # ---- sibling Krylov solvers on the 32x32 system (tol 1e-10): CR and the flexible CG on
    # D^dagger D, BiCGstab-l and the variably preconditioned GCR on D, MinRes on the gauge
    # Laplacian at mass 0.5; preconditioners run on the solve's own operator
    lap5 = Op("laplace", lx, ly, 0.5, U)
    sib = [
        ("cr", normal, {}), ("cr", normal, {"restart_freq": 17}),
        ("minres", lap5, {}), ("minres", lap5, {"omega": 0.8}),
        ("bicgstab_l", stag, {"l": 1}), ("bicgstab_l", stag, {"l": 2}), ("bicgstab_l", stag, {"l": 4}),
        ("bicgstab_l", stag, {"l": 4, "restart_freq": 16}),
        ("fpcg", normal, {"precond": "identity"}), ("fpcg", normal, {"precond": "minres"}),
        ("fpcg", normal, {"precond": "gcr"}), ("fpcg", normal, {"precond": "minres", "restart_freq": 12}),
        ("vpgcr", stag, {"precond": "identity"}), ("vpgcr", stag, {"precond": "minres"}),
        ("vpgcr", stag, {"precond": "gcr"}), ("vpgcr", stag, {"precond": "minres", "restart_freq": 12}),
    ]
    opname = {id(normal): "staggered_normal", id(stag): "staggered", id(lap5): "laplace_m0.5"}
    for solver, op, kw in sib:
        key = "l32_" + solver + "".join(f"_{k}{v}" for k, v in sorted(kw.items()))
        rf = kw.get("restart_freq", 0)
        xs, d, log = R.solve2(solver, op, b, max_iter=10000, eps=1e-10, verbosity=1 if rf == 0 else 2,
                              prefix="[SIB] ", **kw)
        vec[key] = xs
        info["cases"][key] = {**d, "log": log, "solver": solver, "kw": kw, "max_iter": 10000, "eps": 1e-10,
                              "op": opname[id(op)]}
    # detail logs with a max_iter cut, and a preconditioner that prints its own summaries
    for solver, op, kw, mi in (("cr", normal, {}, 6), ("minres", lap5, {}, 5), ("bicgstab_l", stag, {"l": 2}, 6),
                               ("fpcg", normal, {"precond": "minres"}, 4), ("vpgcr", stag, {"precond": "gcr"}, 4)):
        key = f"l32_{solver}_maxiter{mi}"
        _, d, log = R.solve2(solver, op, b, max_iter=mi, eps=1e-10, verbosity=3, prefix="", **kw)
        info["cases"][key] = {**d, "log": log, "solver": solver, "kw": kw, "max_iter": mi,
                              "op": opname[id(op)]}
    _, d, log = R.solve2("fpcg", normal, b, max_iter=3, eps=1e-10, verbosity=3, prefix="[OUT] ",
                         precond="minres", precond_verbosity=1, precond_prefix="  [MR] ")
    info["cases"]["l32_fpcg_precond_log"] = {**d, "log": log, "max_iter": 3, "op": "staggered_normal"}
    # multishift CR on the gauge Laplacian, multishift BiCGstab on D
    for solver, op in (("cr_m", lap), ("bicgstab_m", stag)):
        for rfc, wf in ((1, False), (3, False), (1, True)):
            xs, d, res, log = R.multishift(solver, op, b, msh, resid_freq_check=rfc, max_iter=10000,
                                           eps=1e-10, worst_first=wf, verbosity=1, prefix="[MS] ")
            key = f"l32_{solver}_rfc{rfc}_wf{int(wf)}"
            vec[key] = xs.reshape(-1)
            info["cases"][key] = {**d, "resSqmrhs": res.tolist(), "log": log, "shifts": msh, "rfc": rfc,
                                  "worst_first": wf, "op": "laplace_m0.001" if op is lap else "staggered"}

    # ---- gauge-field utilities (u1_utils.cpp): plaquette, topological charge, a random gauge
    # transform (rand_trans_u1 from mt19937(99)), APE smearing, and the text format of
    # write_gauge_u1 / read_gauge_u1
    for key in ("l32", "l12x6", "g16"):
        lx, ly = (lat[key][0], lat[key][1]) if key in lat else (16, 16)
        U = vec[f"{key}_links"]
        info["cases"][f"{key}_gauge"] = {"plaquette": [R.plaquette(U, lx, ly).real, R.plaquette(U, lx, ly).imag],
                                         "topo": R.topo(U, lx, ly)}
        Ut, g = R.gauge_trans(99, U, lx, ly)
        vec[f"{key}_trans"], vec[f"{key}_links_trans"] = g, Ut
        vec[f"{key}_ape"] = R.ape_smear(U, lx, ly, 0.5, 3)
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        pth = os.path.join(td, "g16.dat")
        R.write_gauge(pth, vec["g16_links"], 16, 16)
        text = open(pth).read()
        vec["g16_links_read"] = R.read_gauge(pth, 16, 16)
    info["cases"]["g16_gauge"]["text"] = text

    # ---- the reference's own heat-bath gauge fields (multigrid/aa_mg/cfg/*.dat, read with
    # read_gauge_u1): beta = 30, and two beta = 60 fields whose file names give their
    # topological charge (q1: +1, qm3: -3).  Smooth fields, unlike rand_gauge_u1's.  Stored: the
    # links as read, the gauge utilities as above, and the reference's CG on the staggered
    # normal equations with the l32 source at m = 0.1 and m = 0.01
    heatbath = {"hb30": "l32t32b30_heatbath.dat", "hb60q1": "l32t32b60_heatbath_q1.dat",
                "hb60qm3": "l32t32b60_heatbath_qm3.dat"}
    for key, fn in heatbath.items():
        U = R.read_gauge(os.path.join(refdir, "multigrid", "aa_mg", "cfg", fn), 32, 32)
        vec[f"{key}_links"] = U
        pl = R.plaquette(U, 32, 32)
        info["cases"][f"{key}_gauge"] = {"plaquette": [pl.real, pl.imag], "topo": R.topo(U, 32, 32),
                                         "file": fn}
        Ut, g = R.gauge_trans(99, U, 32, 32)
        vec[f"{key}_trans"], vec[f"{key}_links_trans"] = g, Ut
        vec[f"{key}_ape"] = R.ape_smear(U, 32, 32, 0.5, 3)
        for tag, m in (("m0.1", 0.1), ("m0.01", 0.01)):
            x, d, _ = R.solve("cg", Op("staggered_normal", 32, 32, m, U), vec["l32_src"], max_iter=10000,
                              eps=1e-10)
            vec[f"{key}_cg_{tag}"] = x
            info["cases"][f"{key}_cg_{tag}"] = {**d, "mass": m, "max_iter": 10000, "eps": 1e-10}

    # ---- multigrid transfer and coarse operators (multigrid/aa_mg/mg_complex.cpp): a 16x16
    # staggered stencil (m = 0.1, plus eo_shift and dof_shift so that the shift projection is
    # exercised) blocked 4x4 with 4 null vectors (Gaussian, numpy seed 5) into a 4x4 lattice
    # with 4 dof; that coarse stencil blocked 2x2 with 4 vectors into 2x2x4; the stencil
    # pieces of the coarse level (tb, bt, m^2 - D_tb D_bt, normal_eo / normal_tb,
    # dagger_eo / dagger_tb) and the top/bottom prepare / reconstruct steps
    rng = np.random.default_rng(5)
    lx, ly = 16, 16
    U16, s16 = R.make_inputs(1337, lx, ly, 1)
    hop, sh = R.staggered_stencil(U16, lx, ly, 0.1, False)
    mgcase = {"lx": lx, "ly": ly, "bx": 4, "by": 4, "nc_c": 4, "shift": [sh.real, sh.imag],
              "eo_shift": [0.03, -0.01], "dof_shift": [0.0, 0.0]}
    vec.update({"mg16_links": U16, "mg16_src": s16[0], "mg16_hop": hop})
    fine = Op("stencil", lx, ly, nc=1, clover=np.zeros(lx * ly, np.complex128), hopping=hop, shift=sh,
              eo_shift=complex(*mgcase["eo_shift"]))
    nv = rng.normal(size=(4, lx * ly)) + 1j * rng.normal(size=(4, lx * ly))
    vec["mg16_nv_in"] = nv.reshape(-1)
    vec["mg16_nv_norm"] = R.mg_block("normalize", lx, ly, 1, 4, 4, 4, nv).reshape(-1)
    P = R.mg_block("orthonormalize", lx, ly, 1, 4, 4, 4, nv)
    vec["mg16_nv_orth"] = P.reshape(-1)
    vc = rng.normal(size=64) + 1j * rng.normal(size=64)
    vec["mg16_coarse_in"] = vc
    vec["mg16_prolong"] = R.mg_prolong(lx, ly, 1, 4, 4, 4, P, vc)
    vec["mg16_restrict"] = R.mg_restrict(lx, ly, 1, 4, 4, 4, P, s16[0])
    for ig in (0, 1):
        cl, hp = R.mg_coarse_stencil(lx, ly, 1, 4, 4, 4, P, fine, bool(ig))
        vec[f"mg16_coarse_clover_ig{ig}"], vec[f"mg16_coarse_hop_ig{ig}"] = cl, hp
    info["cases"]["mg16"] = mgcase
    # second level: the coarse stencil (shifts kept) blocked 2x2 with 4 vectors
    cl, hp = vec["mg16_coarse_clover_ig0"], vec["mg16_coarse_hop_ig0"]
    lev2 = Op("stencil", 4, 4, nc=4, clover=cl, hopping=hp)
    nv2 = rng.normal(size=(4, 64)) + 1j * rng.normal(size=(4, 64))
    vec["mg4_nv_in"] = nv2.reshape(-1)
    P2 = R.mg_block("orthonormalize", 4, 4, 4, 2, 2, 4, nv2)
    vec["mg4_nv_orth"] = P2.reshape(-1)
    vc2 = rng.normal(size=16) + 1j * rng.normal(size=16)
    vec["mg4_coarse_in"] = vc2
    vec["mg4_prolong"] = R.mg_prolong(4, 4, 4, 2, 2, 4, P2, vc2)
    vec["mg4_restrict"] = R.mg_restrict(4, 4, 4, 2, 2, 4, P2, vc)
    vec["mg4_coarse_clover"], vec["mg4_coarse_hop"] = R.mg_coarse_stencil(4, 4, 4, 2, 2, 4, P2, lev2, False)
    # coarse-level stencil pieces on the 4x4x4 stencil with shift 0.1 + 0.02i
    xin = rng.normal(size=64) + 1j * rng.normal(size=64)
    vec["mg16_piece_in"] = xin
    for k in ("stencil_tb", "stencil_bt", "stencil_m2mdtbdbt", "stencil_normal_eo", "stencil_normal_tb",
              "stencil_dagger_eo", "stencil_dagger_tb"):
        vec[f"mg16_{k}"] = R.apply(Op(k, 4, 4, nc=4, clover=cl, hopping=hp, shift=0.1 + 0.02j), xin)
    tbop = Op("stencil_m2mdtbdbt", 4, 4, nc=4, clover=cl, hopping=hp, shift=0.1)
    vec["mg16_tb_prepare"] = R.tbprec(0, tbop, xin)
    vec["mg16_tb_reconstruct"] = R.tbprec(1, tbop, vc, xin)

    # ---- the multigrid preconditioner (mg_complex.cpp:514) inside the variably preconditioned
    # GCR on D, 32x32, m = 0.1: null vectors = 4 Gaussian vectors (numpy seed 11) smoothed by
    # 20 iterations of the reference's CG on D^dagger D, split into even and odd parts (8
    # vectors); 2 levels (4x4 blocks, MinRes smoother 2 + 2, GCR(32) coarse solves to 1e-2,
    # n_max 64) and 3 levels (then 2x2 blocks with 8 Gaussian vectors); 30 outer iterations
    rng = np.random.default_rng(11)
    y_, x_ = np.divmod(np.arange(1024), 32)
    ev = (x_ + y_) % 2 == 0
    sm = []
    for _ in range(4):
        v = rng.normal(size=1024) + 1j * rng.normal(size=1024)
        xs, _, _ = R.solve("cg", normal, v, max_iter=20, eps=1e-30)
        sm.append(xs)
    nv1 = np.concatenate([v * ev for v in sm] + [v * (~ev) for v in sm])
    nv2 = rng.normal(size=8 * 512) + 1j * rng.normal(size=8 * 512)
    vec["mgs_nv1"], vec["mgs_nv2"] = nv1, nv2
    U, b = vec["l32_links"], vec["l32_src"]
    # mgs2: coarse GCR(32) to 1e-2 (n_max 64); mgs2f / mgs3f: fixed coarse work (16 GCR
    # iterations, rel_res 1e-30), a preconditioner that does not depend on where a tolerance
    # test falls
    # mgs3r: the recursive form (MLEVEL_RECURSIVE: the middle level solved by a restarted
    # variably preconditioned GCR, 8 iterations, preconditioned by the level below); mgs3v: a V
    # cycle with no coarse solver (smoothing on every level)
    nv12 = np.concatenate([nv1, nv2])
    for key, blocks, nvecs, nv, n_max, rr, inner, ml in (("mgs2", [4], [8], nv1, 64, 1e-2, 3, 0),
                                                         ("mgs2f", [4], [8], nv1, 16, 1e-30, 3, 0),
                                                         ("mgs3f", [4, 2], [8, 8], nv12, 16, 1e-30, 3, 0),
                                                         ("mgs3r", [4, 2], [8, 8], nv12, 8, 1e-30, 3, 1),
                                                         ("mgs3v", [4, 2], [8, 8], nv12, 8, 1e-30, 0, 0)):
        nr = len(blocks)
        sys.stdout.flush()
        fd, nul = os.dup(1), os.open(os.devnull, os.O_WRONLY)
        os.dup2(nul, 1)  # the reference's mg_preconditioner prints its progress with printf
        try:
            xs, d, log = R.mg_solve("vpgcr", U, 32, 32, 0.1, b, blocks, nvecs, nv, 7, [2] * nr, [2] * nr, inner,
                                    n_max, 32 if ml == 0 else 8, [rr] * nr, mlevel=ml, max_iter=30)
        finally:
            import ctypes
            ctypes.CDLL(None).fflush(None)
            os.dup2(fd, 1)
            os.close(fd)
            os.close(nul)
        vec[f"{key}_solution"] = xs
        summary = [l for l in log.splitlines() if l.startswith("[MGSOLVE]")]
        info["cases"][key] = {**d, "summary": summary[-1], "blocks": blocks, "nvecs": nvecs, "max_iter": 30,
                              "smoother": 7, "n_pre": 2, "n_post": 2, "coarse": inner, "n_max": n_max,
                              "n_restart": 32 if ml == 0 else 8, "rel_res": rr, "mass": 0.1, "mlevel": ml}

    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **vec)
    with open(os.path.join(HERE, "reference_info.json"), "w") as f:
        json.dump(info, f, indent=1, default=lambda o: o.item() if hasattr(o, "item") else str(o))
    print("wrote", len(vec), "vectors")


if __name__ == "__main__":
    main()
