"""Benchmark: time to an FP64-true relative residual of 1e-10 for CG on the staggered normal
equations M^dagger M x = b, 1024x1024 periodic lattice, m = 0.01, U(1) links
exp(i theta) with theta uniform in (-pi, pi) and a complex Gaussian source (std::mt19937 seed
1337, the reference tests' generators), x0 = 0.

One step = one complete solve with the inputs resident in HBM.  The headline arm is the
mixed-precision CG (FP32 inner iterations, FP64 reliable updates); the FP16- and BF16-storage
variants and the plain FP64 GPU CG are timed on the same system and reported beside it.  Between steps the L2 is flushed by writing a 512 MiB buffer (outside the events).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs under torchrun as independent replicas (one system per GPU, no collective on the
data path); rank 0 prints one JSON line.  --impl reference times the reference algorithm on
the host cores (the CPU oracle, a restatement of the reference's CG), rank 0 only.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LX = LY = 1024
MASS = 0.01
EPS = 1e-10
SEED = 1337
MAX_ITER = 100000
# FP64 CG iterations of the reference on this exact system (same generators, same seed),
# measured with the reference's own minv_vector_cg; the GPU FP64 CG reproduces the count.
REF_ITERS = 2093
METRIC = "time-to-1e-10 resid, 1024^2 staggered CG: mixed/batched vs FP64 on GB300; HBM GB/s"
HEADLINE = ("fp32", 1)
# ncu captures of the persistent inner-loop kernels on this workload (profiles/), each stamped
# with the SHA-256 of the kernel's source file when it was captured.  A capture whose stamp no
# longer matches the source is reported as stale (its figures null) rather than applied to a
# changed kernel; tests/test_host_abi.py fails while any stamp is out of date.
#   dram_bytes_per_launch: dram__bytes_read.sum + dram__bytes_write.sum of one launch
#   smem_wavefronts_per_sm_iter: l1tex__data_pipe_lsu_wavefronts_mem_shared.sum over the SMs and
#     the launch's inner iterations (entry included); GB300 serves one 128 B wavefront per clock
#     per SM
CAPTURES = {
    "resident": {"source": "generic-linalg_gb300/csrc/stag_resident.cuh",
                 "sha256": "5cff730dfc24880feeabc9cca4e08fde534ede08f16e7543afee199bca0c321e",
                 "kernel": "k_resident<14, 4, 3> (16 warps, x_lo and links in tensor memory)",
                 "profile": "profiles/k_resident_fp32_1024.md", "iters_per_launch": 20,
                 "dram_bytes_per_launch": 42.142208e6 + 0.022272e6,
                 "smem_wavefronts_per_sm_iter": 18110200 / (152 * 20)},
    "persist": {"source": "generic-linalg_gb300/csrc/stag_tiles.cuh", "sha256": None,
                "kernel": "k_persist", "profile": "profiles/k_persist_fp32_1024.md", "iters_per_launch": 254,
                "dram_bytes_per_launch": 41.987328e6 + 3.212544e6},
}
RESIDENT_CANDIDATES = (6, 7, 8, 11, 12, 13, 14)


def source_sha256(rel):
    import hashlib
    with open(os.path.join(ROOT, rel), "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def capture_for(cand):
    """The ncu capture that describes persistent-kernel candidate `cand`, with "fresh" telling
    whether the kernel source still matches it; None if no capture covers the candidate."""
    key = "resident" if cand in RESIDENT_CANDIDATES else ("persist" if 0 <= cand <= 3 else None)
    if key is None:
        return None
    c = dict(CAPTURES[key])
    c["fresh"] = c["sha256"] is not None and c["sha256"] == source_sha256(c["source"])
    return c


VARIANTS = [("fp32", 1), ("fp16", 2), ("bf16", 3)]
# persistent inner-loop kernels by the library's candidate index (glinalg_tuned_persist)
PERSIST_KERNELS = {0: "k_persist<16 warps, 4 rows>", 1: "k_persist<16 warps, 8 rows>",
                   2: "k_persist<32 warps, 2 rows>", 3: "k_persist<16 warps, 2 rows>",
                   4: "k_persist_bulk<256x4 tiles>", 5: "k_persist_bulk<512x2 tiles>",
                   6: "k_resident<16 warps, x_lo in registers> (rectangle state on chip)",
                   7: "k_resident<32 warps> (rectangle state on chip)",
                   8: "k_resident<16 warps> (rectangle state on chip)",
                   9: "k_resident1<16 warps> (single-reduction form)",
                   10: "k_resident1<32 warps> (single-reduction form)",
                   11: "k_resident<16 warps, x_lo in tensor memory> (rectangle state on chip)",
                   12: "k_resident<32 warps, x_lo in tensor memory> (rectangle state on chip)",
                   13: "k_resident<16 warps, x_lo and links in tensor memory> (rectangle state on chip)",
                   14: "k_resident<32 warps, x_lo and links in tensor memory> (rectangle state on chip)",
                   15: "k_resident_s<16 warps, 16-bit p' and t> (rectangle state on chip, t = D p' each iteration)"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# The workload both arms are quoted on (printed as `config` by each).
CONFIG = {"workload": "staggered normal-equation CG to FP64-true relres 1e-10, 1024x1024, m=0.01, x0=0",
          "lattice": [LX, LY], "mass": MASS, "tol": EPS, "max_iter": MAX_ITER,
          "inputs": "std::mt19937(1337): rand_gauge_u1 links (theta uniform in (-pi, pi)), then a "
                    "gaussian complex source"}


def oracle_inputs():
    """Links and source from the oracle's own restatement of the reference tests' generators
    (std::mt19937(1337), rand_gauge_u1, then gaussian): no library code involved."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    g = pyoracle.Generator(SEED)
    U = g.rand_gauge_u1(LX, LY)
    b = g.gaussian(LX * LY)
    return U, b


def oracle_solve(U, b, threads=None):
    """One complete FP64 CG solve of the workload by the CPU oracle (the reference's
    minv_vector_cg, generic_cg.cpp:278-382, restated; operator and vector loops spread over
    `threads` host threads, sums serial in the reference's order, so the iterates are the
    serial reference's bit for bit).  Returns (x, info, seconds, threads used)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    O = pyoracle.Oracle()
    nth = O.set_threads(threads)
    op = pyoracle.Operator("staggered_normal", LX, LY, MASS, U)
    t0 = time.perf_counter()
    x, info, _ = O.solve("cg", op, b, max_iter=MAX_ITER, eps=EPS)
    dt = time.perf_counter() - t0
    return x, info, dt, nth


def cpu_sample_text(info, nth):
    return (f"one complete solve per step: {info['iter']} CG iterations, {info['ops_count']} operator "
            f"applications, true relres {np.sqrt(info['resSq']) / BNORM[0]:.3e}; operator and vector "
            f"loops on {nth} host threads, dot and norm sums serial in the reference's order")


BNORM = [1.0]


def run_reference(args):
    """--impl reference: the reference's CG (the oracle port: oracle/_ref needs the reference
    checkout, absent on the GPU machine) on the host cores, W + K complete solves of the workload;
    rank 0 only.  Loads only the oracle's library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    U, b = oracle_inputs()
    BNORM[0] = float(np.linalg.norm(b))
    samples, info, nth = [], None, 1
    for i in range(args.warmup + args.steps):
        _, info, dt, nth = oracle_solve(U, b)
        if not info["success"]:
            raise RuntimeError(f"reference CG did not converge: {info}")
        if i >= args.warmup:
            samples.append(dt * 1e3)
    v = statistics.mean(samples)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(v, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": CONFIG,
        "variant": "fp64 CG (the reference's algorithm on the host cores)",
        "results": {"iters": info["iter"], "ops_count": info["ops_count"],
                    "true_relres_fp64": float(np.sqrt(info["resSq"]) / BNORM[0]),
                    "ms_min_max": [round(min(samples), 3), round(max(samples), 3)]},
        "cpu_baseline": {"value": round(v, 3), "unit": "ms", "cores": nth, "kind": "port",
                         "sample": cpu_sample_text(info, nth)},
        "e2e": {"value": round(v, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def kernels_only(args):
    """The headline variant's inner-iteration kernels on the 1024x1024 lattice, n launches
    each (steps), timed with CUDA events; about 60 MB on the device."""
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    L = gl.lib()
    g = gl.Generator(SEED)
    U = g.rand_gauge_u1(LX, LY)
    op = gl.Operator(2, LX, LY, MASS, torch.from_numpy(U).cuda())
    kms = (C_double * 2)()
    kbytes = (C_double * 2)()
    gl._capi.check(L.glinalg_profile_mixed_kernels(op.handle, HEADLINE[1], max(1, args.steps), kms, kbytes),
                   "profile")
    for nm, j in (("A", 0), ("B", 1)):
        print(json.dumps({"kernel": nm, "variant": HEADLINE[0], "ms": kms[j], "bytes": kbytes[j],
                          "GB/s": kbytes[j] / (kms[j] * 1e-3) / 1e9}))


def probe_solve(args):
    """One solve of the 1024x1024 system in the variant --probe-variant (the headline's by
    default) stopped after --probe-iters inner iterations: one launch of the persistent
    inner-loop kernel, a small case for ncu captures."""
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    g = gl.Generator(SEED)
    U = g.rand_gauge_u1(LX, LY)
    b = g.gaussian(LX * LY)
    op = gl.Operator(2, LX, LY, MASS, torch.from_numpy(U).cuda())
    bd = torch.from_numpy(b).cuda()
    x = torch.zeros_like(bd)
    prec = dict([HEADLINE] + VARIANTS + [("fp64", 0)])[args.probe_variant]
    info = gl.minv_vector_cg(x, bd, bd.numel(), args.probe_iters, EPS, gl.square_staggered_normal_u1, op,
                             precision=prec)
    print(json.dumps({"probe": f"{args.probe_variant} variant, 1024x1024", "iters": info.iter,
                      "kernel_launches": info.kernel_launches, "kernel_ms": info.kernel_ms}))


def _flush_and_time(fn, flush, stream):
    """fn() between CUDA events on `stream`, after writing the L2-flush buffer."""
    import torch
    flush.fill_(1.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def workload_multishift(args):
    """Multishift CG on the staggered normal equations, 512x512, m = 0.05, 12 shifts log-spaced
    over [1e-4, 1], tolerance 1e-10 per shift: one source and 64 sources in one batched solve
    (glinalg_cg_m_multi), FP64 (the reference's recurrence) and mixed precision (FP32
    multishift with FP64 scalar recurrences, then every shift refined by the mixed CG to an
    FP64-true 1e-10), against 64 single-source FP64 solves one after another.  Inputs from
    std::mt19937(1337): links, then the sources in order."""
    import numpy as np
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    replicas = importlib.import_module("generic-linalg_gb300.replicas")
    rank, world, local = dist_setup()
    L = gl.lib()
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    gl._capi.check(L.glinalg_set_stream(C_void(stream.cuda_stream), 1), "set_stream")
    lx = ly = 512
    mass = 0.05
    n_all, shifts = args.sources, np.logspace(-4, 0, 12)
    g = gl.Generator(SEED)
    U = g.rand_gauge_u1(lx, ly)
    B_all = np.stack([g.gaussian(lx * ly) for _ in range(n_all)])
    # under torchrun every rank takes an equal share of the sources (no collective on the data
    # path); source 0 stays on rank 0, where the oracle checks it
    mine = replicas.my_share([1.0] * n_all, rank, world)
    B = B_all[mine]
    n_rhs = len(mine)
    op = gl.Operator(2, lx, ly, mass, torch.from_numpy(U).to(dev))
    Bd = torch.from_numpy(B).to(dev)
    X = torch.zeros((n_rhs, len(shifts), lx * ly), dtype=torch.complex128, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    Ax = torch.zeros(lx * ly, dtype=torch.complex128, device=dev)

    def true_relres(xq, q, sg):
        op.apply(Ax, xq)
        return float(torch.linalg.vector_norm(Bd[q] - Ax - sg * xq) / torch.linalg.vector_norm(Bd[q]))

    out, sol0 = {}, {}
    for name, prec in [v for v in (("fp64", 0), ("fp32", 1)) if v[0] in args.ms_variants.split(",")]:
        res = {}
        for nr in (1, n_rhs):
            for i in range(args.warmup + args.steps):
                X.zero_()
                if world > 1:
                    torch.distributed.barrier()
                t, infos = _flush_and_time(
                    lambda: gl.cg_m_multi(op, X[:nr], Bd[:nr], shifts, 1, 100000, 1e-10, precision=prec),
                    flush, stream)
                if i >= args.warmup:
                    res.setdefault(nr, []).append(replicas.max_over_ranks(t, world, dev) if nr == n_rhs else t)
            assert all(inf.success for inf in infos), (name, infos)
            res[f"info{nr}"] = infos
        i64 = res[f"info{n_rhs}"]
        ms64 = statistics.mean(res[n_rhs])
        worst = max(true_relres(X[q, k], q, sg) for q in (0, n_rhs - 1) for k, sg in enumerate(shifts))
        sol0[name] = X[0].cpu().numpy().copy()
        out[name] = {"one_source_ms": round(statistics.mean(res[1]), 3), "one_source_iters": res["info1"][0].iter,
                     "batched_multishift_phase_ms": round(i64[0].kernel_ms, 3) if prec else None,
                     "batched_ms": round(ms64, 3), "batched_ms_per_source": round(ms64 / n_rhs, 3),
                     "batched_iters_min_max": [min(i.iter for i in i64), max(i.iter for i in i64)],
                     "operator_applications_per_source_mean": round(statistics.mean(i.ops_count for i in i64), 1),
                     "batched_algorithmic_GBps": round(sum(i.gbytes for i in i64) / (ms64 * 1e-3), 1),
                     "max_shift_true_relres_sources_0_and_63": worst}
    # the same 64 sources, one single-source FP64 solve after another (one GPU)
    t_seq = None
    if world == 1 and not args.no_one_by_one:
        xs = [torch.zeros(lx * ly, dtype=torch.complex128, device=dev) for _ in shifts]

        def one_by_one():
            for q in range(n_rhs):
                gl.minv_vector_cg_m(xs, Bd[q], len(shifts), lx * ly, 1, 100000, 1e-10, shifts.copy(),
                                    gl.square_staggered_normal_u1, op)
        t_seq, _ = _flush_and_time(one_by_one, flush, stream)
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    line = {"workload": "multishift CG, staggered normal equations 512x512, m=0.05, 12 shifts logspace[1e-4,1], tol 1e-10",
            "steps": args.steps, "warmup": args.warmup, "l2": "flushed (512 MiB write) before every solve",
            "sources": n_all, "n_gpus": world, "scaling": "strong",
            "parallelism": f"replicas x{world} (sources shared out, no collective on the data path)",
            "variants": out, "fp64_one_by_one_ms": round(t_seq, 3) if t_seq else None,
            "mixed_speedup_vs_fp64_batched": (round(out["fp64"]["batched_ms"] / out["fp32"]["batched_ms"], 2)
                                              if len(out) == 2 else None),
            "mixed_speedup_vs_fp64_one_by_one": (round(t_seq / out["fp32"]["batched_ms"], 2)
                                                 if t_seq and "fp32" in out else None)}
    if not args.no_cpu_baseline:
        # the oracle's CG-M (the reference's recurrence, site loops on every host core) on source 0:
        # one complete solve, and every variant's source-0 solutions against it
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        O = pyoracle.Oracle()
        nth = O.set_threads(None)
        oop = pyoracle.Operator("staggered_normal", lx, ly, mass, U)
        t0 = time.perf_counter()
        xo, io, _ = O.cg_m(oop, B[0], shifts, max_iter=100000, eps=1e-10)
        dt = time.perf_counter() - t0
        for name in out:
            out[name]["source0_max_shift_err_vs_oracle"] = float(max(
                np.linalg.norm(sol0[name][k] - xo[k]) / np.linalg.norm(xo[k]) for k in range(len(shifts))))
        line["cpu_baseline"] = {"value": round(dt * 1e3 * n_all, 1), "unit": "ms (64 sources)", "cores": nth,
                                "kind": "port",
                                "sample": f"one complete CG-M solve of source 0 ({io['iter']} iterations, "
                                          f"{dt:.2f} s on {nth} threads) times 64 sources"}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def dist_setup():
    """(rank, world, local rank) from torchrun's environment; the NCCL process group is made
    only for more than one rank (the systems are shared out, no collective on the data path)."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl")
    return rank, world, local


def workload_batch(args):
    """256 independent systems in one batch: sides from {32, 64, 128, 256}, links U(1) random,
    masses log-uniform in [0.01, 0.5]; even systems staggered D^dagger D (mass m), odd systems
    the gauge Laplacian (mass m^2); FP32 inner iterations with FP64 reliable updates, tolerance
    1e-10.  One batched call (glinalg_cg_batch) against one mixed solve per system.  Under
    torchrun every rank solves its share (replicas.shard_by_cost, cost = sites / mass, about
    sites x sqrt(kappa)) in one batched call; the job's time is the slowest rank's."""
    import numpy as np
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    replicas = importlib.import_module("generic-linalg_gb300.replicas")
    rank, world, local = dist_setup()
    L = gl.lib()
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    gl._capi.check(L.glinalg_set_stream(C_void(stream.cuda_stream), 1), "set_stream")
    g = gl.Generator(2024)
    rng = np.random.default_rng(2024)
    meta, host = [], []
    for q in range(args.systems):
        side = int(rng.choice([32, 64, 128, 256]))
        m = float(np.exp(rng.uniform(np.log(0.01), np.log(0.5))))
        kind = 2 if q % 2 == 0 else 3
        U = g.rand_gauge_u1(side, side)
        b = g.gaussian(side * side)
        meta.append((kind, side, m if kind == 2 else m * m, m))
        host.append((U, b))
    mine = replicas.my_share([side * side / m for _, side, _, m in meta], rank, world)
    ops, bs, xs = [], [], []
    for q in mine:
        kind, side, mass, _ = meta[q]
        U, b = host[q]
        ops.append(gl.Operator(kind, side, side, mass, torch.from_numpy(U).to(dev)))
        bs.append(torch.from_numpy(b).to(dev))
        xs.append(torch.zeros(side * side, dtype=torch.complex128, device=dev))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    times = []
    for i in range(args.warmup + args.steps):
        for x in xs:
            x.zero_()
        if world > 1:
            torch.distributed.barrier()
        t, infos = _flush_and_time(lambda: gl.cg_batch(ops, xs, bs, 100000, 1e-10, precision=1), flush, stream)
        if i >= args.warmup:
            times.append(replicas.max_over_ranks(t, world, dev))
    assert all(inf.success for inf in infos)
    results = replicas.gather_results({q: (inf.iter, inf.gbytes) for q, inf in zip(mine, infos)}, world)
    assert sorted(results) == list(range(args.systems))

    def one_by_one():
        for q in range(len(ops)):
            cb = gl.square_staggered_normal_u1 if meta[mine[q]][0] == 2 else gl.square_laplace_u1
            gl.minv_vector_cg(xs[q], bs[q], xs[q].numel(), 100000, 1e-10, cb, ops[q], precision=1)
    t_seq = None
    if world == 1 and not args.no_one_by_one:
        for x in xs:
            x.zero_()
        one_by_one()
        for x in xs:
            x.zero_()
        t_seq, _ = _flush_and_time(one_by_one, flush, stream)
    ms = statistics.mean(times)
    sites = sum(s * s for _, s, _, _ in meta)
    if rank == 0:
        its = [it for it, _ in results.values()]
        line = {"workload": f"{args.systems} uneven systems (sides 32..256, half staggered normal, half Laplacian), FP32 inner + FP64 reliable, tol 1e-10",
                "steps": args.steps, "warmup": args.warmup, "sites": sites, "n_gpus": world,
                "parallelism": f"replicas x{world} (systems shared out by cost, no collective on the data path)",
                "scaling": "strong", "l2": "flushed (512 MiB write) before every solve",
                "batched_ms": round(ms, 3), "iters_min_max": [min(its), max(its)],
                "one_by_one_ms": round(t_seq, 3) if t_seq else None,
                "batch_speedup": round(t_seq / ms, 2) if t_seq else None,
                "algorithmic_GBps": round(sum(gb for _, gb in results.values()) / (ms * 1e-3), 1)}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def workload_siblings(args):
    """The reference's sibling Krylov solvers (FP64, the reference's recurrences) on one
    256x256 system from std::mt19937(1337): CR, CR-M (12 shifts logspace[1e-4, 1]) and the
    flexibly preconditioned CG (MinRes(4) preconditioner) on D^dagger D with m = 0.05;
    BiCGstab-2, BiCGstab-4, BiCGstab-M and the variably preconditioned GCR (MinRes(4)) on D;
    MinRes on the gauge Laplacian with mass 0.5.  Tolerance 1e-10; device-resident fields, L2
    flushed before every solve.  The CPU baseline is the oracle's same solver on the same
    system for a few iterations, extrapolated linearly to the GPU's iteration count."""
    import numpy as np
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    L = gl.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    gl._capi.check(L.glinalg_set_stream(C_void(stream.cuda_stream), 1), "set_stream")
    lx = ly = 256
    g = gl.Generator(SEED)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(lx * ly)
    Ud, bd = torch.from_numpy(U).to(dev), torch.from_numpy(b).to(dev)
    nrm = gl.StaggeredU1Op(Ud, 0.05, lx, ly)
    lap = gl.StaggeredU1Op(Ud, 0.5, lx, ly)
    N, D, LAP = gl.square_staggered_normal_u1, gl.square_staggered_u1, gl.square_laplace_u1
    shifts = np.logspace(-4, 0, 12)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    x = torch.zeros_like(bd)
    xs = [torch.zeros_like(bd) for _ in shifts]
    n = lx * ly
    cases = {
        "CR": lambda: gl.minv_vector_cr(x, bd, n, 100000, EPS, N, nrm),
        "MinRes (Laplacian, mass 0.5)": lambda: gl.minv_vector_minres(x, bd, n, 100000, EPS, 1.0, LAP, lap),
        "BiCGStab-2": lambda: gl.minv_vector_bicgstab_l(x, bd, n, 100000, EPS, 2, D, nrm),
        "BiCGStab-4": lambda: gl.minv_vector_bicgstab_l(x, bd, n, 100000, EPS, 4, D, nrm),
        "FPCG, MinRes(4) preconditioner": lambda: gl.minv_vector_cg_flex_precond(
            x, bd, n, 100000, EPS, N, nrm, gl.minres_preconditioner, gl.MinresPrecondStruct(4, 0.1, N, nrm)),
        "VPGCR, MinRes(4) preconditioner": lambda: gl.minv_vector_gcr_var_precond(
            x, bd, n, 100000, EPS, D, nrm, gl.minres_preconditioner, gl.MinresPrecondStruct(4, 0.1, D, nrm)),
        "CR-M (12 shifts)": lambda: gl.minv_vector_cr_m(xs, bd, 12, n, 1, 100000, EPS, shifts.copy(), N, nrm),
        "BiCGstab-M (12 shifts)": lambda: gl.minv_vector_bicgstab_m(xs, bd, 12, n, 1, 100000, EPS, shifts.copy(),
                                                                    D, nrm),
    }
    out = {}
    for name, fn in cases.items():
        ts, info = [], None
        for i in range(args.warmup + args.steps):
            x.zero_()
            t, info = _flush_and_time(fn, flush, stream)
            if i >= args.warmup:
                ts.append(t)
        ms = statistics.mean(ts)
        out[name] = {"ms": round(ms, 3), "iters": info.iter, "ops": info.ops_count, "success": info.success,
                     "algorithmic_GBps": round(info.gbytes / (ms * 1e-3), 1)}
    line = {"workload": "sibling Krylov solvers, 256x256, m=0.05 (Laplacian mass 0.5), tol 1e-10, FP64",
            "steps": args.steps, "warmup": args.warmup, "l2": "flushed (512 MiB write) before every solve",
            "solvers": out}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        O = pyoracle.Oracle()
        on = pyoracle.Operator("staggered_normal", lx, ly, 0.05, U)
        od = pyoracle.Operator("staggered", lx, ly, 0.05, U)
        ol = pyoracle.Operator("laplace", lx, ly, 0.5, U)
        samples = {"CR": ("cr", on, {}), "MinRes (Laplacian, mass 0.5)": ("minres", ol, {}),
                   "BiCGStab-2": ("bicgstab_l", od, {"l": 2}), "BiCGStab-4": ("bicgstab_l", od, {"l": 4}),
                   "FPCG, MinRes(4) preconditioner": ("fpcg", on, {"precond": "minres", "rel_res": 0.1}),
                   "VPGCR, MinRes(4) preconditioner": ("vpgcr", od, {"precond": "minres", "rel_res": 0.1})}
        cpu = {}
        for name, (solver, oop, kw) in samples.items():
            k = 8 if solver != "bicgstab_l" else 8 * kw["l"]
            t0 = time.perf_counter()
            O.solve2(solver, oop, b, max_iter=k, eps=EPS, **kw)
            dt = time.perf_counter() - t0
            cpu[name] = round(dt / k * out[name]["iters"] * 1e3, 1)
        line["cpu_baseline"] = {"unit": "ms per solve", "cores": 1, "kind": "port", "values": cpu,
                                "sample": "8 iterations (BiCGStab-l: 8 cycles) of the oracle's same solver on "
                                          "the same system, extrapolated linearly to the GPU's iteration count "
                                          "(an underestimate for FPCG / VPGCR, whose cost per iteration grows)"}
    print(json.dumps(line))


def workload_rows(args):
    """Measurements of the rows beyond the headline at 1024x1024 (links and source from
    std::mt19937(1337)), L2 flushed before every timed call, device-resident fields:
    even/odd preconditioning (prepare, the FP64 and FP32 CG on m^2 - D_eo D_oe to 1e-10,
    reconstruct); the multigrid transfers of a 4x4-blocked level with 8 null vectors (prolong,
    restrict, block orthonormalisation, the Galerkin coarse stencil and its apply); the gauge
    utilities (plaquette, gauge transform, one APE sweep).  Algorithmic bytes count every array
    read or written once; GB/s against the measured HBM copy bandwidth."""
    import numpy as np
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    L = gl.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    gl._capi.check(L.glinalg_set_stream(C_void(stream.cuda_stream), 1), "set_stream")
    lx = ly = 1024
    n = lx * ly
    g = gl.Generator(SEED)
    U = g.rand_gauge_u1(lx, ly)
    b = g.gaussian(n)
    Ud, bd = torch.from_numpy(U).to(dev), torch.from_numpy(b).to(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    hbm = peaks()[0]

    def timed(fn, reps=None):
        ts, out = [], None
        for i in range(args.warmup + (reps or args.steps)):
            t, out = _flush_and_time(fn, flush, stream)
            if i >= args.warmup:
                ts.append(t)
        return statistics.mean(ts), out

    def rate(nbytes, ms):
        return {"ms": round(ms, 4), "GBps": round(nbytes / (ms * 1e-3) / 1e9, 1),
                "frac_of_hbm": round(nbytes / (ms * 1e-3) / 1e9 / hbm, 3)}

    out = {}
    # even/odd preconditioning (f1)
    eo = gl.Operator(9, lx, ly, 0.01, Ud)
    rhs_e = torch.zeros_like(bd)
    ms, _ = timed(lambda: gl.square_staggered_eoprec_prepare(rhs_e, bd, eo))
    out["eo_prepare"] = rate(16.0 * n * 4, ms)  # rhs, two links, rhs_e
    for prec, nm in (() if args.rows_kernels else ((0, "eo_cg_fp64"), (1, "eo_cg_fp32_reliable"))):
        xe = torch.zeros_like(bd)

        def solve():
            xe.zero_()
            return gl.minv_vector_cg(xe, rhs_e, n, 100000, EPS, gl.square_staggered_m2mdeodoe_u1, eo, precision=prec)
        ms, info = timed(solve, reps=max(1, min(args.steps, 3)))
        out[nm] = {"ms": round(ms, 3), "iters": info.iter, "success": info.success, "solver": info.name,
                   "reliable_updates": info.reliable_updates, "inner_kernel_ms": round(info.kernel_ms, 3),
                   "algorithmic_GBps": round(info.gbytes / (ms * 1e-3), 1)}
    full = torch.zeros_like(bd)
    if args.rows_kernels:
        xe = rhs_e
    ms, _ = timed(lambda: gl.square_staggered_eoprec_reconstruct(full, xe, bd, eo))
    out["eo_reconstruct"] = rate(16.0 * n * 5, ms)
    # multigrid transfers (f2): 4x4 blocks, 8 vectors -> 256x256x8
    nc = 8
    nv = torch.from_numpy(np.stack([g.gaussian(n) for _ in range(nc)])).to(dev)
    lv = gl.MgLevel(lx, ly, 1, 4, 4, nc, nv)
    csize = (lx // 4) * (ly // 4) * nc
    ms, _ = timed(lambda: gl.block_orthonormalize(lv), reps=3)
    out["mg_block_orthonormalize"] = rate(16.0 * n * nc * 4, ms)  # (nc-1) passes read+write ~ 2 r/w per vector
    vc = torch.from_numpy(g.gaussian(csize)).to(dev)
    fine = torch.zeros_like(bd)
    ms, _ = timed(lambda: gl.prolong(fine, vc, lv))
    out["mg_prolong"] = rate(16.0 * (n * nc + n + csize), ms)
    coarse = torch.zeros_like(vc)
    ms, _ = timed(lambda: gl.restrict(coarse, bd, lv))
    out["mg_restrict"] = rate(16.0 * (n * nc + n + csize), ms)
    st = gl.Stencil2D(lx, ly, 1, shift=0.01)
    gl.get_square_staggered_u1_stencil(st, gl.StaggeredU1Op(U, 0.01, lx, ly))
    fop = gl.Operator(4, lx, ly, nc=1, clover=st.clover, hopping=st.hopping, shift=st.shift)
    ms, cop = timed(lambda: gl.generate_coarse_from_fine_stencil(None, fop, lv), reps=3)
    out["mg_coarse_stencil"] = rate(16.0 * (n * nc + 5 * n + 5 * (csize // nc) * nc * nc), ms)
    cin = torch.from_numpy(g.gaussian(csize)).to(dev)
    cout = torch.zeros_like(cin)
    ms, _ = timed(lambda: cop.apply(cout, cin))
    out["mg_coarse_apply_256x256x8"] = rate(16.0 * (2 * csize + 5 * (csize // nc) * nc * nc), ms)
    # gauge utilities (f4)
    ms, _ = timed(lambda: gl.get_plaquette_u1(Ud, lx, ly))
    out["plaquette"] = rate(16.0 * 2 * n, ms)
    gt = torch.from_numpy(g.rand_trans_u1(lx, ly)).to(dev)
    Uw = Ud.clone()
    ms, _ = timed(lambda: gl.apply_gauge_trans_u1(Uw, gt, lx, ly))
    out["gauge_trans"] = rate(16.0 * (4 * n + n), ms)
    Us = torch.zeros_like(Ud)
    ms, _ = timed(lambda: gl.apply_ape_smear_u1(Us, Ud, lx, ly, 0.5, 1))
    out["ape_smear_1_sweep"] = rate(16.0 * 2 * n * 2 * 2, ms)  # copy in, sweep (read + write), copy out
    line = {"workload": "rows beyond the headline, 1024x1024, m = 0.01", "steps": args.steps,
            "warmup": args.warmup, "l2": "flushed (512 MiB write) before every call", "hbm_peak_GBps": hbm,
            "rows": out}
    if not args.no_cpu_baseline and not args.rows_kernels:
        # the oracle (the reference's algorithms restated in C, one core) on the same inputs
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        O = pyoracle.Oracle()

        def cpu(fn):
            t0 = time.perf_counter()
            r_ = fn()
            return (time.perf_counter() - t0) * 1e3, r_

        cpu_ms = {}
        oeo = pyoracle.Operator("staggered_m2mdeodoe", lx, ly, 0.01, U)
        cpu_ms["eo_prepare"], rhs_h = cpu(lambda: O.eoprec_prepare(oeo, b))
        t10, _ = cpu(lambda: O.solve("cg", oeo, rhs_h, max_iter=10, eps=EPS))
        cpu_ms["eo_cg_fp64"] = t10 / 10 * out["eo_cg_fp64"]["iters"]
        cpu_ms["eo_reconstruct"], _ = cpu(lambda: O.eoprec_reconstruct(oeo, rhs_h, b))
        nvh = nv.cpu().numpy()
        cpu_ms["mg_block_orthonormalize"], P = cpu(lambda: O.mg_block("orthonormalize", lx, ly, 1, 4, 4, nc, nvh))
        vch = vc.cpu().numpy()
        cpu_ms["mg_prolong"], _ = cpu(lambda: O.mg_prolong(lx, ly, 1, 4, 4, nc, P, vch))
        cpu_ms["mg_restrict"], _ = cpu(lambda: O.mg_restrict(lx, ly, 1, 4, 4, nc, P, b))
        ofine = pyoracle.Operator("stencil", lx, ly, nc=1, clover=st.clover, hopping=st.hopping, shift=st.shift)
        # the probing of generate_coarse_from_fine_stencil on a 256x256 block of the same form,
        # scaled by the site count
        lx4 = 256
        U4 = U.reshape(ly, lx, 2)[:lx4, :lx4].reshape(-1)
        st4 = gl.Stencil2D(lx4, lx4, 1, shift=0.01)
        gl.get_square_staggered_u1_stencil(st4, gl.StaggeredU1Op(U4, 0.01, lx4, lx4))
        o4 = pyoracle.Operator("stencil", lx4, lx4, nc=1, clover=st4.clover, hopping=st4.hopping, shift=st4.shift)
        P4 = P.reshape(nc, ly, lx)[:, :lx4, :lx4].reshape(nc, -1)
        t4, _ = cpu(lambda: O.mg_coarse_stencil(lx4, lx4, 1, 4, 4, nc, P4, o4))
        cpu_ms["mg_coarse_stencil"] = t4 * (n / (lx4 * lx4))
        del ofine
        import ctypes
        cl_h = np.zeros((csize // nc) * nc * nc, np.complex128)
        hp_h = np.zeros(4 * (csize // nc) * nc * nc, np.complex128)
        L.glinalg_operator_stencil_get(cop.handle, cl_h.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       hp_h.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0)
        oc = pyoracle.Operator("stencil", lx // 4, ly // 4, nc=nc, clover=cl_h, hopping=hp_h)
        cpu_ms["mg_coarse_apply_256x256x8"], _ = cpu(lambda: O.apply(oc, cin.cpu().numpy()))
        cpu_ms["plaquette"], _ = cpu(lambda: O.plaquette(U, lx, ly))
        cpu_ms["gauge_trans"], _ = cpu(lambda: O.gauge_trans(U, gt.cpu().numpy(), lx, ly))
        cpu_ms["ape_smear_1_sweep"], _ = cpu(lambda: O.ape_smear(U, lx, ly, 0.5, 1))
        line["cpu_baseline"] = {"unit": "ms per call", "cores": 1, "kind": "port",
                                "values": {k: round(v, 3) for k, v in cpu_ms.items()},
                                "sample": "the oracle on the same inputs, one call each; the FP64 even/odd CG "
                                          "from 10 iterations scaled to the GPU's count; the coarse-stencil "
                                          "probing on a 256x256 corner scaled by the site count"}
    print(json.dumps(line))


def workload_eo(args):
    """Even/odd solve of M x = b (M = m + D, the staggered operator) on the 1024x1024, m = 0.01
    system of the headline, by the reference's recipe (tests/staggered_pieces/staggered_pieces.cpp:
    331-346): prepare rhs_e = m b_e - D_eo b_o, CG on m^2 - D_eo D_oe to 1e-10, reconstruct
    x_o = (b_o - D_oe x_e) / m.  GPU: the checkerboarded FP32 CG with FP64 reliable updates,
    device-resident fields (L2 flushed before every step), and end to end through the public API
    from pinned host buffers (the operator built from host links once per step).  Inputs from
    the oracle's generator (std::mt19937(1337)); the solution is checked against the oracle's
    FP64 even/odd solve, whose time on the host threads is the CPU baseline."""
    import numpy as np
    import torch
    gl = importlib.import_module("generic-linalg_gb300")
    L = gl.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    gl._capi.check(L.glinalg_set_stream(C_void(stream.cuda_stream), 1), "set_stream")
    U, b = oracle_inputs()
    n = LX * LY
    Ud, bd = torch.from_numpy(U).to(dev), torch.from_numpy(b).to(dev)
    eo = gl.Operator(9, LX, LY, MASS, Ud)
    rhs_e, xe, x = torch.zeros_like(bd), torch.zeros_like(bd), torch.zeros_like(bd)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        gl.square_staggered_eoprec_prepare(rhs_e, bd, eo)
        xe.zero_()
        info = gl.minv_vector_cg(xe, rhs_e, n, MAX_ITER, EPS, gl.square_staggered_m2mdeodoe_u1, eo, precision=1)
        gl.square_staggered_eoprec_reconstruct(x, xe, bd, eo)
        return info

    clocks = ClockSampler(0)
    for _ in range(args.warmup):
        _flush_and_time(step, flush, stream)
    clocks.start()
    times, infos = [], []
    for _ in range(args.steps):
        t, info = _flush_and_time(step, flush, stream)
        times.append(t)
        infos.append(info)
    clk = clocks.stop()
    info = infos[-1]
    if not info.success:
        raise RuntimeError(f"even/odd solve did not converge: {info}")
    Mx = torch.zeros_like(bd)
    gl.Operator(0, LX, LY, MASS, Ud).apply(Mx, x)
    relres = (torch.linalg.vector_norm(bd - Mx) / torch.linalg.vector_norm(bd)).item()
    xg = x.cpu().numpy()

    # end to end: host links and fields, copies inside the timed region
    Uh = torch.from_numpy(U).pin_memory().numpy()
    bh = torch.from_numpy(b).pin_memory().numpy()
    rh, xeh, xh = (torch.zeros(n, dtype=torch.complex128).pin_memory().numpy() for _ in range(3))
    e2e = []
    for i in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op_h = gl.Operator(9, LX, LY, MASS, Uh)
        gl.square_staggered_eoprec_prepare(rh, bh, op_h)
        xeh[:] = 0
        inf_h = gl.minv_vector_cg(xeh, rh, n, MAX_ITER, EPS, gl.square_staggered_m2mdeodoe_u1, op_h, precision=1)
        gl.square_staggered_eoprec_reconstruct(xh, xeh, bh, op_h)
        op_h.close()
        if i >= args.warmup:
            e2e.append((time.perf_counter() - t0) * 1e3)
        assert inf_h.success
    field = 16 * n
    line = {"workload": "even/odd solve of M x = b (prepare, CG on m^2 - D_eo D_oe to 1e-10, reconstruct), "
                        "1024x1024, m=0.01, checkerboarded FP32 CG with FP64 reliable updates",
            "metric": "even/odd solve time", "value": round(statistics.mean(times), 3), "unit": "ms",
            "higher_is_better": False, "steps": args.steps, "warmup": args.warmup, "dtype": "fp32 (FP64 reliable)",
            "data": "synthetic: std::mt19937(1337) links and gaussian source (the oracle's generator)",
            "l2": "flushed (512 MiB write) before every step",
            "e2e": {"value": round(statistics.mean(e2e), 3), "unit": "ms",
                    "h2d_bytes_per_step": 2 * field + field + 2 * field + 2 * field,
                    "d2h_bytes_per_step": 3 * field},
            "results": {"solver": info.name, "inner_iters": info.iter, "reliable_updates": info.reliable_updates,
                        "inner_kernel_ms": round(info.kernel_ms, 3),
                        "inner_us_per_iter": round(1e3 * info.kernel_ms / max(1, info.iter), 3),
                        "true_relres_full_system_fp64": relres,
                        "ms_min_max": [round(min(times), 3), round(max(times), 3)]},
            "clocks": clk}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        O = pyoracle.Oracle()
        nth = O.set_threads(None)
        oeo = pyoracle.Operator("staggered_m2mdeodoe", LX, LY, MASS, U)
        t0 = time.perf_counter()
        rhs_o = O.eoprec_prepare(oeo, b)
        xo_e, oinfo, _ = O.solve("cg", oeo, rhs_o, max_iter=MAX_ITER, eps=EPS)
        x_or = O.eoprec_reconstruct(oeo, xo_e, b)
        cpu_ms = (time.perf_counter() - t0) * 1e3
        line["results"]["oracle_iters"] = oinfo["iter"]
        line["results"]["err_vs_oracle"] = float(np.linalg.norm(xg - x_or) / np.linalg.norm(x_or))
        line["cpu_baseline"] = {"value": round(cpu_ms, 3), "unit": "ms", "cores": nth, "kind": "port",
                                "sample": f"one complete FP64 even/odd solve (prepare, {oinfo['iter']} CG iterations, "
                                          f"reconstruct) by the oracle, operator and vector loops on {nth} host "
                                          f"threads, sums serial in the reference's order"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--ref-iters", type=int, default=30)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sources", type=int, default=64, help="multishift workload: sources (64)")
    ap.add_argument("--ms-variants", default="fp64,fp32", help="multishift workload: fp64 and/or fp32")
    ap.add_argument("--systems", type=int, default=256, help="batch workload: systems (256)")
    ap.add_argument("--no-one-by-one", action="store_true",
                    help="batched workloads: skip the one-call-per-system comparison")
    ap.add_argument("--variants", default="fp32,fp16,bf16,fp64",
                    help="comma list of the variants to time besides the headline (fp32)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="only time the two inner-iteration kernels of the headline variant "
                         "(a small case for ncu captures)")
    ap.add_argument("--rows-kernels", action="store_true",
                    help="rows workload: the kernels only (no solves, no CPU baseline), for a launch list")
    ap.add_argument("--workload", default="headline",
                    choices=["headline", "multishift", "batch", "siblings", "rows", "eo"],
                    help="multishift / batch: time the batched workloads instead (one JSON line each)")
    ap.add_argument("--probe-variant", default="fp32", choices=["fp32", "fp16", "bf16", "fp64"],
                    help="the variant of the --probe-iters solve")
    ap.add_argument("--probe-iters", type=int, default=0,
                    help="run one headline-variant solve stopped after this many inner iterations "
                         "(one persistent-kernel launch; a small case for ncu captures) and exit")
    args = ap.parse_args()
    if args.probe_iters > 0 and args.impl == "ours":
        return probe_solve(args)
    if args.workload == "multishift" and args.impl == "ours":
        return workload_multishift(args)
    if args.workload == "batch" and args.impl == "ours":
        return workload_batch(args)
    if args.workload == "siblings" and args.impl == "ours":
        return workload_siblings(args)
    if args.workload == "rows" and args.impl == "ours":
        return workload_rows(args)
    if args.workload == "eo" and args.impl == "ours":
        return workload_eo(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.kernels_only:
        return kernels_only(args)

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    gl = importlib.import_module("generic-linalg_gb300")
    L = gl.lib()
    # a dedicated (non-default) stream shared by torch and the library, so that the CUDA
    # events below bracket exactly the library's work
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    gl._capi.check(L.glinalg_set_stream(C_void(stream.cuda_stream), 1), "set_stream")

    # inputs: every replica solves the same seeded system (the work per GPU is fixed)
    g = gl.Generator(SEED)
    U = g.rand_gauge_u1(LX, LY)
    b = g.gaussian(LX * LY)
    Ud = torch.from_numpy(U).to(dev)
    bd = torch.from_numpy(b).to(dev)
    op = gl.Operator(2, LX, LY, MASS, Ud)
    x = torch.zeros_like(bd)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def solve(prec):
        x.zero_()
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        info = gl.minv_vector_cg(x, bd, bd.numel(), MAX_ITER, EPS, gl.square_staggered_normal_u1, op,
                                 precision=prec)
        e1.record(stream)
        torch.cuda.synchronize()
        if not info.success and prec == HEADLINE[1]:
            raise RuntimeError(f"headline solve did not converge: {info}")
        return e0.elapsed_time(e1), info

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    results, sols = {}, {}
    clocks = ClockSampler(local)
    head_name, head_prec = HEADLINE
    wanted = set(args.variants.split(","))
    for name, prec in [HEADLINE] + [v for v in VARIANTS if v != HEADLINE and v[0] in wanted]:
        for _ in range(args.warmup):
            solve(prec)
        barrier()
        if name == head_name:
            clocks.start()
        times, infos = [], []
        for _ in range(args.steps):
            t, info = solve(prec)
            times.append(t)
            infos.append(info)
        barrier()
        if name == head_name:
            clk = clocks.stop()
        results[name] = (times, infos)
        sols[name] = x.cpu().numpy().copy()
    # the plain FP64 GPU CG (reference recurrence) on the same system
    if "fp64" in wanted:
        solve(0)
        t64 = [solve(0) for _ in range(max(1, args.fp64_steps))]
        results["fp64"] = ([t for t, _ in t64], [i for _, i in t64])
        sols["fp64"] = x.cpu().numpy().copy()

    head_times, head_infos = results[head_name]
    ms = statistics.mean(head_times)
    ms_max = ms
    if dist:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_max = tt.item()

    # true residual of the headline solution, rechecked with the FP64 operator
    xh_head = torch.from_numpy(sols[head_name]).to(dev)
    Ax = torch.zeros_like(bd)
    op.apply(Ax, xh_head)

    # dominant kernel: the persistent inner-loop kernel of the headline solve (both stencil
    # phases, the vector updates and the grid-wide sums), timed with CUDA events around launches
    # of its own on the library stream, each running the timed solve's mean inner iterations per
    # launch; cross-checked with the kernel's device clock inside the timed solves
    hbm_peak, peak_src = peaks()
    hi_ = head_infos[-1]
    k_launch = max(1, hi_.kernel_launches)
    persist_cand = L.glinalg_tuned_persist(op.handle, head_prec)
    persist_kernel = PERSIST_KERNELS.get(persist_cand, "none")
    resident = persist_cand in RESIDENT_CANDIDATES
    # algorithmic bytes: the canonical CG iteration on D^dagger D, 17 complex words per site
    # (D p -> t: p, 2 links, t; D^dagger t -> Ap: t, 2 links, Ap; x, p, r, Ap in, x, r out;
    # p = r + beta p: 3), 136 B per site in FP32
    cg_bytes = 17 * 8.0 * LX * LY
    k_ms_solve = hi_.kernel_ms / k_launch
    it_per_launch = max(1, round(hi_.iter / k_launch))
    ev_ms, ev_bytes, ev_cand = C_double(), C_double(), C_int()
    gl._capi.check(L.glinalg_profile_persist_kernel(op.handle, head_prec, 5, it_per_launch, ev_ms, ev_bytes,
                                                    ev_cand), "profile_persist_kernel")
    k_ms, k_bytes = ev_ms.value, cg_bytes * it_per_launch
    hbm_equiv = k_bytes / (k_ms * 1e-3) / 1e9
    hbm_equiv_solve = (cg_bytes * hi_.iter / k_launch / (k_ms_solve * 1e-3) / 1e9) if k_ms_solve > 0 else 0.0
    smem_gbs, smem_ms = C_double(), C_double()
    gl._capi.check(L.glinalg_probe_smem_bandwidth(smem_gbs, smem_ms), "probe_smem_bandwidth")
    # the probe can not exceed what the SMs' shared-memory ports serve (128 B per clock per SM)
    n_sm0 = torch.cuda.get_device_properties(dev).multi_processor_count
    smem_arch = 128.0 * n_sm0 * 2070e6 / 1e9
    assert smem_gbs.value <= 1.05 * smem_arch, (smem_gbs.value, smem_arch)

    # e2e through the public API with host buffers (pinned), copies inside the timed region
    Uh = torch.from_numpy(U).pin_memory().numpy()
    bh = torch.from_numpy(b).pin_memory().numpy()
    xh = torch.zeros(LX * LY, dtype=torch.complex128).pin_memory().numpy()
    e2e_times = []
    for i in range(args.warmup + args.steps):
        xh[:] = 0
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        info = gl.minv_vector_cg(xh, bh, bh.size, MAX_ITER, EPS, gl.square_staggered_normal_u1,
                                 gl.StaggeredU1Op(Uh, MASS, LX, LY), precision=head_prec)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append((time.perf_counter() - t0) * 1e3)
        assert info.success
    e2e_ms = statistics.mean(e2e_times)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    hi = head_infos[-1]
    t64m = statistics.mean(results["fp64"][0]) if "fp64" in results else float("nan")
    relres = (torch.linalg.vector_norm(bd - Ax) / torch.linalg.vector_norm(bd)).item()
    # the FP64 CPU oracle's solution of the same system (its own generator, bit-identical inputs):
    # the CPU baseline and the reference point of every variant's solution error
    cb, x_or, or_info = None, None, None
    if not args.no_cpu_baseline:
        Uo, bo = oracle_inputs()
        assert np.array_equal(Uo, U) and np.array_equal(bo, b), "oracle and library generators disagree"
        BNORM[0] = float(np.linalg.norm(bo))
        x_or, or_info, dt, nth = oracle_solve(Uo, bo)
        cb = {"value": round(dt * 1e3, 3), "unit": "ms", "cores": nth, "kind": "port",
              "sample": cpu_sample_text(or_info, nth)}
    variants = {}
    for name in [n for n in ("fp32", "fp16", "bf16", "fp64") if n in results]:
        ts, ins = results[name]
        variants[name] = {"ms": round(statistics.mean(ts), 3), "iters": ins[-1].iter,
                          "converged": bool(ins[-1].success),
                          "reliable_updates": ins[-1].reliable_updates,
                          "true_relres": float(np.sqrt(ins[-1].resSq) / np.linalg.norm(b)),
                          "gbytes": round(ins[-1].gbytes, 3)}
        if x_or is not None:
            variants[name]["err_vs_oracle"] = float(np.linalg.norm(sols[name] - x_or) / np.linalg.norm(x_or))
    # kernels of one headline solve: link packing, |b|^2 and the setup reliable update (6),
    # then per cycle of the outer loop the persistent inner-loop kernel, the reliable update
    # (6), the outer-loop tail and the graph's loop guard
    launches = 8 + 9 * hi.kernel_launches
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    roof = {"kernel": f"{persist_kernel} ({head_name}; inner CG iterations: D p, D^dagger t, updates, "
                      "2 grid-wide sums)",
            "bytes_per_launch": k_bytes, "ms_per_launch": round(k_ms, 4), "iters_per_launch": it_per_launch,
            "launches_per_solve": hi_.kernel_launches,
            "share_of_solve": round(hi_.kernel_ms / hi_.device_ms, 3) if hi_.device_ms else None,
            "timing": "CUDA events on the library stream around 5 launches of the kernel, each running the "
                      "timed solve's mean inner iterations per launch",
            "hbm_equivalent_gbs": round(hbm_equiv, 1),
            "hbm_equivalent_note": "136 B per site and inner iteration (the CG iteration on D^dagger D as 17 "
                                   "complex FP32 words per site: D p -> t: 4; D^dagger t -> Ap: 4; x, p, r, Ap "
                                   "in, x, r out: 6; p = r + beta p: 3) over the kernel's time: the rate any "
                                   "HBM-streaming iteration would need to match it; its fields stay on chip",
            "hbm_equivalent_gbs_in_solve": round(hbm_equiv_solve, 1),
            "hbm_peak_gbs": hbm_peak, "hbm_peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"}
    cap = capture_for(persist_cand)
    if resident:
        # the iteration's fields never leave the SM: the binding resource is shared memory.
        # achieved = shared-memory wavefronts (128 B each, from the ncu capture of this kernel
        # source) per launch over the launch's CUDA-event time; peak = the probe's measured rate
        fresh = cap is not None and cap["fresh"]
        smem_bytes = cap["smem_wavefronts_per_sm_iter"] * 128.0 * n_sm * it_per_launch if fresh else None
        smem_ach = smem_bytes / (k_ms * 1e-3) / 1e9 if smem_bytes else None
        roof.update({
            "bound": "smem", "unit": "GB/s", "peak": round(smem_gbs.value, 1),
            "achieved": round(smem_ach, 1) if smem_ach else None,
            "frac": round(smem_ach / smem_gbs.value, 3) if smem_ach else None,
            "peak_source": "measured in this run: glinalg_probe_smem_bandwidth (conflict-free 128-bit "
                           "shared-memory loads, 2 x 1024 threads per SM)",
            "achieved_note": "128 B x shared-memory wavefronts per SM and inner iteration (ncu capture of this "
                             "kernel source, profiles/k_resident_fp32_1024.md) x SMs x iterations per launch, "
                             "over the launch's CUDA-event time",
            "traffic": cap["dram_bytes_per_launch"] if fresh else None,
            "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one launch (ncu capture of this "
                            "kernel source): the entry load of the launch's state; it does not grow with "
                            "its iterations",
            "capture": {k: v for k, v in (cap or {}).items() if k != "fresh"} or None,
            "capture_matches_source": fresh})
    else:
        fresh = cap is not None and cap["fresh"]
        roof.update({"bound": "hbm", "unit": "GB/s", "achieved": round(hbm_equiv, 1), "peak": hbm_peak,
                     "frac": round(hbm_equiv / hbm_peak, 3), "peak_source": roof["hbm_peak_source"],
                     "traffic": cap["dram_bytes_per_launch"] if fresh else None,
                     "capture_matches_source": fresh})
    line = {
        "metric": METRIC, "value": round(ms_max, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (inner iterations; fp64 reliable updates and solution)",
        "data": "synthetic (seeded U(1) links and Gaussian source, std::mt19937 1337)",
        "config": CONFIG,
        "variant": f"{head_name} inner + fp64 reliable updates",
        "parallelism": f"replicas x{world}", "l2": "flushed (512 MiB write) before every step",
        "results": {"inner_iters": hi.iter, "reliable_updates": hi.reliable_updates,
                    "true_relres_fp64": relres,
                    "err_vs_oracle": variants.get(head_name, {}).get("err_vs_oracle"),
                    "oracle_iters": or_info["iter"] if or_info else None,
                    "fp64_gpu_ms": round(t64m, 3), "speedup_vs_fp64_gpu": round(t64m / ms, 2),
                    "variants": variants},
        "roofline": roof,
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": int(Uh.nbytes + bh.nbytes + xh.nbytes),
                "d2h_bytes_per_step": int(xh.nbytes)},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if cb:
        line["cpu_baseline"] = cb
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


from ctypes import c_double as C_double, c_int as C_int, c_void_p as C_void  # noqa: E402

if __name__ == "__main__":
    main()
