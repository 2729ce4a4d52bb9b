"""Benchmark: pressure-correction PCG solves/s on GB300 (one JSON line).

Workload (one "step"): one Jacobi-PCG solve of the pressure-correction (p')
system of a jittered mixed triangle/quad mesh of the unit square,
1672 x 1672 quads of which a seeded half are split (4,19x,xxx cells), nodes
jittered by uniform +-20% of the edge (seed 1234), RCM-ordered, assembled
on the GPU (CellibPressure.f coefficients, one cell pinned), stored CSRD
(the reference's matriz 1), RHS uniform[-1,1] (seed 42), x0 = 0, solved to
||b - A x||2 / ||b||2 <= 1e-8 (recomputed in FP64).

value   solves/s of the mixed-precision path (FP32 CG inside FP64 defect
        correction), inputs resident in HBM, CUDA events on the solve stream.
e2e     the same solve through the public host API (solver(), the
        reference's argument list) with pinned host arrays: matrix values,
        b and x copied in and x copied out inside the timed region.
Also reported: the plain FP64 persistent PCG (same stopping rule) solves/s,
the FP64 SpMV GB/s, and the CPU restatement of the reference's OpenMP PCG
(pcg_omp + matvec_csrd_omp + dot_ompL4) timed on this host's cores.

--impl reference times only that CPU restatement (the reference is Fortran
and cannot be built here), on the same workload and metric.
"""
from __future__ import annotations

import argparse
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

TOL = 1e-8
C4_TOL = 1e-8
NX_DEFAULT = 1672
L2_BYTES = 129 * 1024 * 1024


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)
            if self._stop.is_set():
                break

    def stop(self) -> dict:
        self._stop.set()
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        smax = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(self.samples)}


def build_mesh(nx: int):
    from fortranfvcell_gb300 import mesh
    return mesh.square_mesh(nx, kind="mixed", jitter=0.2, seed=1234)


def build_system_gpu(nx: int):
    """Product setup chain: host C++ graph tools + GPU assembly."""
    from fortranfvcell_gb300 import mesh
    t0 = time.time()
    m = build_mesh(nx)
    s = mesh.pressure_system(m, matriz=1, unsym=True, pin_cell=1)
    b = np.random.default_rng(42).uniform(-1.0, 1.0, s.neq)
    log(f"setup: {s.neq} cells, nad {s.nad}, {time.time() - t0:.1f} s")
    return s, b


def pcg_bytes_fp64(n, nnz):
    # SpMV (12 B per true off-diagonal + 24 B per row) + 11 vector streams
    return 12 * nnz + 24 * n + 11 * 8 * n


def cg_bytes_fp32(n, nnz):
    # one mixed-precision CG iteration: a 4-byte weight and a 2-byte column
    # offset per true off-diagonal; phase A reads z and the p_prev pair and
    # writes the p pair and q (24 B per row); phase B reads q, the residual
    # pair and 1/m and writes the residual pair and z (28 B per row), and
    # every second iteration reads the correction pair and both p pairs and
    # writes the correction pair (32 B, 16 per iteration)
    return 6 * nnz + 68 * n


# DRAM bytes per mixed-CG iteration measured with ncu on the profiling case
# of this workload (bench.py --profile-its 200: dram__bytes_read.sum +
# dram__bytes_write.sum of mixed_cg_staged_w4, less its three FP64 residual
# sweeps, / 200); used to report roofline.traffic, scaled by the iterations
# of a launch.
MEASURED_BYTES_PER_ITERATION = {4192598: 402.0e6}
MEASURED_BYTES_PER_SWEEP = {4192598: 0.33e9}


def refine_bytes(n, nnz):
    # FP64 residual sweep (SpMV + b read + scaled residual write) and the
    # FP64 correction pass (x, D^-1/2, e read; x written)
    return 12 * nnz + 24 * n + 8 * n + 4 * n + 28 * n


def oracle_whole_solve(ad, au, ia, ja, n, nad, b, threads):
    """One whole solve by the CPU restatement of the reference's OpenMP PCG
    (pcg_omp + matvec_csrd_omp + dot_ompL4, Iterativos_omp.f:30-127) from
    x = 0, stopped on ||r|| <= TOL ||b|| -- the rule the GPU solves use --
    timed.  Returns (x, iterations, seconds, FP64-recomputed relres)."""
    import scipy.sparse as sp
    from oracle import oracle
    x = np.zeros(n)
    t0 = time.perf_counter()
    rc, so = oracle.pcg_omp_sample(ad, au, x, b.copy(), ia, ja, n, nad, TOL, 200000, 1, threads,
                                   stop_rule=1)
    el = time.perf_counter() - t0
    rows = np.repeat(np.arange(n), np.diff(ia))
    A = sp.csr_matrix((au[:nad], (rows, ja[:nad] - 1)), shape=(n, n)) + sp.diags(ad)
    rel = float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))
    return x, int(so.iterations), el, rel, int(rc)


def oracle_s_per_iteration(ad, au, ia, ja, n, nad, b, threads, its, matriz=1):
    """Seconds per iteration of the reference's own pcg_omp loop (its
    stopping test, run past convergence), over `its` iterations; matriz 1
    (CSRD, matvec_csrd_omp) or 4 (ELLPACK, matvec_ellpack_omp)."""
    from oracle import oracle
    x = np.zeros(n)
    t0 = time.perf_counter()
    oracle.pcg_omp_sample(ad, au, x, b.copy(), ia, ja, n, nad, 1e-300, its, matriz, threads)
    return (time.perf_counter() - t0) / its


def cpu_sample(s, b, one_thread_s=3.0):
    """The CPU restatement of the reference's OpenMP PCG on this host: one
    whole solve on all host threads (its time is the baseline, no
    extrapolation), and a 1-thread sample of iterations scaled by the whole
    solve's iteration count."""
    threads = os.cpu_count() or 1
    n = s.neq
    x, its, el, rel, rc = oracle_whole_solve(s.ad, s.au, s.ia, s.ja, n, s.nad, b, threads)
    per1 = oracle_s_per_iteration(s.ad, s.au, s.ia, s.ja, n, s.nad, b, 1, 3)
    k1 = int(max(3, min(2000, one_thread_s / max(per1, 1e-6))))
    per1 = oracle_s_per_iteration(s.ad, s.au, s.ia, s.ja, n, s.nad, b, 1, k1)
    out = {"value": 1.0 / el, "unit": "solves/s", "cores": threads, "kind": "port",
           "sample": f"one whole pcg_omp solve (matvec_csrd_omp, dot_ompL4) of the {n}-row "
                     f"system from x = 0 to ||r|| <= {TOL:g} ||b||: {its} iterations in "
                     f"{el:.1f} s on {threads} threads",
           "iterations": its, "whole_solve_s": round(el, 3), "rel_residual_fp64": rel,
           "s_per_iteration": el / its,
           "one_thread": {"value": 1.0 / (per1 * its), "unit": "solves/s", "cores": 1,
                          "sample": f"{k1} pcg_omp iterations on 1 thread "
                                    f"({per1 * 1e3:.2f} ms each) x {its} iterations per solve"}}
    return out, x


def run_ours(args):
    import torch
    import fortranfvcell_gb300 as fvc
    from fortranfvcell_gb300 import Context, make_opts

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    s, b = build_system_gpu(args.nx)
    n = s.neq
    stream = torch.cuda.Stream()
    ctx = Context(device=local, stream=stream)
    ctx.set_matrix(1, True, n, s.nad, s.ad, s.au, s.au, s.ia, s.ja)
    info = ctx.info()
    nnz = info["nnz_off"]
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    o_mixed = make_opts("mixed", init=1, refine_tol=TOL, inner_tol=args.inner_tol)
    o_fp64 = make_opts("fp64", init=1, stop_rule=1)

    def solve(opts, which):
        with torch.cuda.stream(stream):
            st = ctx.solve(1, bd, xd, TOL, 200000, opts)
        return st

    # warm-up
    for _ in range(args.warmup):
        st_m = solve(o_mixed, "mixed")
    A_rel = None

    def true_rel():
        x = xd.cpu().numpy()
        import scipy.sparse as sp
        r = np.repeat(np.arange(n), np.diff(s.ia))
        A = sp.csr_matrix((s.au, (r, s.ja - 1)), shape=(n, n)) + sp.diags(s.ad)
        return float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))

    # timed region: mixed precision (the headline)
    launches0 = fvc.kernel_launches()
    clk = ClockSampler(local)
    clk.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stats = []
    for _ in range(args.steps):
        stats.append(solve(o_mixed, "mixed"))
    ev1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = clk.stop()
    launches = fvc.kernel_launches() - launches0
    ms_total = ev0.elapsed_time(ev1)
    if ws > 1:
        t = torch.tensor([ms_total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / args.steps
    rel_mixed = true_rel()
    st = stats[-1]
    kernel_ms = statistics.mean(x.solve_ms for x in stats)
    inner = st.inner_iterations
    sweeps = st.refinements
    alg_bytes = inner * cg_bytes_fp32(n, nnz) + (sweeps + 1) * refine_bytes(n, nnz)
    traffic = None
    if n in MEASURED_BYTES_PER_ITERATION:
        traffic = int(inner * MEASURED_BYTES_PER_ITERATION[n]
                      + (sweeps + 1) * MEASURED_BYTES_PER_SWEEP[n])
    hbm, peak_kind = peaks()
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9

    # plain FP64 persistent PCG, same stopping rule
    st64 = solve(o_fp64, "fp64")
    rel64 = true_rel()
    x64 = xd.cpu().numpy()
    t64 = [solve(o_fp64, "fp64").solve_ms for _ in range(max(1, min(2, args.steps)))]
    ms64 = statistics.mean(t64)
    fp64_bytes = st64.iterations * pcg_bytes_fp64(n, nnz)

    # FP64 SpMV GB/s: the fused kernel the solvers run, and the kernel with
    # the reference's separate rounding (bit-identical to Matvec.f)
    y = torch.empty_like(bd)

    def time_spmv(fn, reps=20):
        for _ in range(3):
            fn(bd, y)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn(bd, y)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    spmv_ms = time_spmv(ctx.spmv_fast)
    spmv_ref_ms = time_spmv(ctx.spmv)
    spmv_bytes = 12 * nnz + 24 * n
    spmv_gbs = spmv_bytes / (spmv_ms * 1e-3) / 1e9
    # the FP32 operator of the mixed solves (difference form, built by them):
    # a 4-byte weight and a 16-bit column offset per true off-diagonal, e, x
    # and y per row.  Only true nonzeros count: the padding slots of the
    # triangle rows (stored to width 4) are overhead
    x32 = bd.float()
    y32 = torch.empty_like(x32)
    spmv32_ms = time_spmv(lambda xv, yv: ctx.spmv_f32(x32, y32))
    inf = ctx.info()
    spmv32_bytes = 6 * nnz + 12 * n
    spmv32_gbs = spmv32_bytes / (spmv32_ms * 1e-3) / 1e9

    # the launch-shape autotuner on this matrix: its pick against the
    # automatic shape, per iteration over the same trial length
    tuned = {}
    for name, code, prec in (("pcg_fp64", 1, "fp64"), ("pcg_mixed", 1, "mixed")):
        o_best, us_best = ctx.autotune(code, prec, 50)
        o_def = make_opts(prec, init=1)
        xt = torch.zeros_like(bd)
        ctx.solve(code, bd, xt, 1e-300, 50, o_def, raise_on_error=False)
        st_def = ctx.solve(code, bd, xt, 1e-300, 50, o_def, raise_on_error=False)
        us_def = st_def.solve_ms * 1e3 / max(st_def.iterations, 1)
        tuned[name] = {"block_threads": o_best.block_threads, "max_blocks": o_best.max_blocks,
                       "staging": o_best.staging, "us_per_iteration": round(us_best, 2),
                       "automatic_us_per_iteration": round(us_def, 2)}

    # end to end through the public host API, pinned host arrays
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h_ad, h_au, h_b = pin(s.ad), pin(s.au), pin(b)
    h_ia, h_ja = pin(s.ia), pin(s.ja)
    h_x = pin(np.zeros(n))
    o_e2e = make_opts("mixed", init=1, refine_tol=TOL, inner_tol=args.inner_tol)
    fvc.solver(h_ad, h_au, h_au, h_x, h_b, h_ia, h_ja, n, s.nad, True, TOL, 200000, 1, 1,
               opts=o_e2e)  # structure upload (cached afterwards)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(3, args.steps))
    for _ in range(e2e_steps):
        h_x[:] = 0.0
        fvc.solver(h_ad, h_au, h_au, h_x, h_b, h_ia, h_ja, n, s.nad, True, TOL, 200000, 1, 1,
                   opts=o_e2e)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = h_ad.nbytes + h_au.nbytes + h_b.nbytes + h_x.nbytes
    d2h = h_x.nbytes

    if ws > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return None
    cpu, fp64_vs_oracle = None, None
    if not args.no_cpu:
        cpu, x_cpu = cpu_sample(s, b)
        # the 4M FP64 solve on both sides under one rule (||r|| <= 1e-8 ||b||
        # from x = 0): iteration counts and the distance between solutions
        fp64_vs_oracle = {"rule": f"||r|| <= {TOL:g} ||b||, x0 = 0",
                          "gpu_iterations": int(st64.iterations),
                          "oracle_iterations": cpu["iterations"],
                          "x_rel_l2": float(f"{np.linalg.norm(x64 - x_cpu) / np.linalg.norm(x_cpu):.3e}"),
                          "oracle": "pcg_omp (Iterativos_omp.f:30-127) restated, OpenMP"}
    value = ws * 1000.0 / ms_step
    line = {
        "metric": "PCG solves/s to ||b-Ax||/||b||<=1e-8, p' system, mixed FP32/FP64 "
                  "(plain FP64 and SpMV GB/s alongside)",
        "value": round(value, 4),
        "unit": "solves/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32-inner/f64-refine",
        "data": "synthetic",
        "config": {"workload": f"p' Jacobi-PCG, jittered mixed tri/quad unit square, {n} cells "
                               f"(nx={args.nx}), RCM, CSRD -> SELL-32, b~U[-1,1] seed 42, x0=0",
                   "cells": n, "nnz_off": nnz, "tol_rel_residual": TOL,
                   "l2": "inputs larger than L2 (working set > 129 MB), no flush",
                   "parallelism": f"replicas x{ws}"},
        "solve": {"mixed": {"solves_per_s": round(1000.0 / ms_step, 4),
                            "inner_iterations": inner, "refinements": sweeps,
                            "rel_residual_fp64": rel_mixed, "kernel_ms": round(kernel_ms, 3)},
                  "fp64": {"solves_per_s": round(1000.0 / ms64, 4),
                           "iterations": st64.iterations, "rel_residual_fp64": rel64,
                           "kernel_ms": round(ms64, 3),
                           "gbs": round(fp64_bytes / (ms64 * 1e-3) / 1e9, 1),
                           "vs_oracle": fp64_vs_oracle},
                  "mixed_over_fp64": round(ms64 / ms_step, 3)},
        "spmv": {"gbs": round(spmv_gbs, 1), "ms": round(spmv_ms, 4), "bytes": spmv_bytes,
                 "frac_of_peak": round(spmv_gbs / hbm, 3),
                 "ref_rounding_gbs": round(spmv_bytes / (spmv_ref_ms * 1e-3) / 1e9, 1),
                 "bound": "FP64 issue rate (FP64 pipe ~75% active), not HBM",
                 "fp32": {"gbs": round(spmv32_gbs, 1), "ms": round(spmv32_ms, 4),
                          "bytes": spmv32_bytes, "frac_of_peak": round(spmv32_gbs / hbm, 3),
                          "kernel": "spmv_f32, the mixed solves' operator"}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(achieved / hbm, 3), "traffic": traffic,
                     "kernel": "mixed_cg (persistent, one launch per solve)",
                     "peak_kind": peak_kind,
                     "alg_bytes_per_launch": int(alg_bytes)},
        "autotune": tuned,
        "e2e": {"value": round(1.0 / e2e_s, 4), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0 and not args.no_simple:
        line["simple_c1"] = run_simple_c1(args)
    if rank == 0 and not args.no_c2:
        line["standalone_c2"] = run_c2(args)
    if rank == 0 and args.c4_cases > 0:
        line["batched_c4"] = run_batched_c4(args)
    if rank == 0 and args.c3_nx > 0:
        line["gas_c3"] = run_gas_c3(args)
    if rank == 0 and args.c5_nx > 0:
        line["adjoint_c5"] = run_adjoint_c5(args)
    return line


def run_simple_c1(args):
    """The C1 configuration: the Re = 100 lid-driven cavity on 64 x 64 quads,
    200 SIMPLE outer iterations (u, v BiCGSTAB on ELLPACK, p' PCG on CSRD,
    tolerances 1e-8, underU 0.7, underPc 0.3, steady).  GPU: the
    device-resident loop (cells.SimpleLoop), wall time.  CPU: the same
    iteration restated over the oracle (sequential solvers, one core)."""
    from fortranfvcell_gb300.cases import lid_driven_cavity
    from fortranfvcell_gb300.cells import SimpleLoop
    case = lid_driven_cavity(args.simple_nx)
    nit = args.simple_its
    loop = SimpleLoop(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                      case["sedge"], case["e"])
    loop.iterate(2)                       # warm-up: kernels and solver scratch
    loop.set_fields(np.zeros((case["numel"], 2)), np.zeros(case["numel"]))
    loop.close()
    loop = SimpleLoop(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                      case["sedge"], case["e"])
    t0 = time.perf_counter()
    res, its = loop.iterate(nit)
    gpu_s = time.perf_counter() - t0
    w, _ = loop.fields()
    loop.close()
    # the same iterations as one CUDA graph launch each (captured before the clock)
    loop = SimpleLoop(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                      case["sedge"], case["e"])
    loop.use_graph(True)
    t0 = time.perf_counter()
    loop.iterate(0)
    capture_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    res_g, its_g = loop.iterate(nit)
    graph_s = time.perf_counter() - t0
    w_g, _ = loop.fields()
    loop.close()
    out = {"workload": f"lid-driven cavity Re={1.0 / case['e'][0, 0]:g}, {args.simple_nx}x"
                       f"{args.simple_nx} quads, {nit} SIMPLE outer iterations",
           "gpu_s": round(gpu_s, 4), "outer_its_per_s": round(nit / gpu_s, 2),
           "graph": {"gpu_s": round(graph_s, 4), "outer_its_per_s": round(nit / graph_s, 2),
                     "capture_s": round(capture_s, 4),
                     "same_as_uncaptured": bool(np.array_equal(res_g, res)
                                                and np.array_equal(its_g, its)
                                                and np.array_equal(w_g, w))},
           "solver_iterations": [int(v) for v in its.sum(axis=0)],
           "final_residuals": [float(f"{v:.3e}") for v in res[-1]],
           "u_min_centreline": float(np.round(np.min(0.5 * (
               w[:, 0].reshape(args.simple_nx, -1)[:, args.simple_nx // 2 - 1]
               + w[:, 0].reshape(args.simple_nx, -1)[:, args.simple_nx // 2])), 4))}
    if not args.no_cpu:
        from oracle import oracle
        from oracle.simple_ref import SimpleRef
        ref = SimpleRef(oracle, case)
        t0 = time.perf_counter()
        for _ in range(nit):
            ref.step()
        cpu_s = time.perf_counter() - t0
        out["cpu_port_s"] = round(cpu_s, 4)
        out["cpu_kind"] = "port (restated reference, sequential solvers, 1 core)"
        out["max_abs_w_difference"] = float(f"{np.abs(w - ref.w).max():.2e}")
    return out


def run_gas_c3(args):
    """The C3 configuration: natural convection in a differentially heated
    square cavity, ideal-gas SIMPLE loop with the energy equation (air,
    Pr 0.72, dT 1 K around 20 C, adiabatic top and bottom, side set for
    Ra = 1e6) on nx x nx quads, steady pseudo-time (dt 1e10), underU 0.7,
    underPc 0.3, from rest at 20 C.  GPU: the device-resident loop with FP64
    solves and with mixed FP32/FP64 solves, the same outer iterations;
    per-field differences of the mixed run against the FP64 one.  CPU: the
    same iteration restated (sequential solvers, one core), a bounded
    sample of outer iterations."""
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts

    def loop_for(case, prec):
        # mixed: the FP32-inner solves for p' and, with c3_precision_u
        # mixed, for momentum and enthalpy
        pu = args.c3_precision_u if prec == "mixed" else "fp64"
        lp = SimpleLoop(case["coor"], case["ix"], case["nelcon"], case["num"], case["pedge"],
                        case["sedge"], case["e"],
                        opts=simple_opts(precision=prec, precision_u=pu))
        lp.enable_energy(case["pedgeE"], case["sedgeE"], case["gravity"], case["t0"])
        return lp

    warm = natural_convection_cavity(32, ra=args.c3_ra)
    for prec in ("fp64", "mixed"):
        lp = loop_for(warm, prec)
        lp.iterate_energy(3)
        lp.close()
    c = natural_convection_cavity(args.c3_nx, ra=args.c3_ra)
    nit = args.c3_its
    out = {"workload": f"natural convection, ideal gas + energy, {args.c3_nx}x{args.c3_nx} quads "
                       f"({c['numel']} cells), Ra={args.c3_ra:g}, steady pseudo-time, "
                       f"{nit} outer iterations from rest"}
    fields = {}
    for prec in ("fp64", "mixed"):
        lp = loop_for(c, prec)
        t0 = time.perf_counter()
        res, its = lp.iterate_energy(nit)
        el = time.perf_counter() - t0
        w, p = lp.fields()
        t, _, _ = lp.energy_fields()
        lp.close()
        fields[prec] = (w, p, t)
        out[prec] = {"gpu_s": round(el, 3), "outer_its_per_s": round(nit / el, 2),
                     "solver_iterations": [int(v) for v in its.sum(axis=0)],
                     "final_residuals": [float(f"{v:.3e}") for v in res[-1]]}
    (w64, p64, t64), (wmx, pmx, tmx) = fields["fp64"], fields["mixed"]
    out["mixed_vs_fp64"] = {
        "w_rel_max": float(f"{np.abs(wmx - w64).max() / np.abs(w64).max():.2e}"),
        "p_rel_max": float(f"{np.abs(pmx - p64).max() / max(np.abs(p64).max(), 1e-300):.2e}"),
        "t_max_K": float(f"{np.abs(tmx - t64).max():.2e}")}
    if not args.no_cpu:
        from oracle import oracle
        from oracle.simple_ref import GasSimpleRef
        ref = GasSimpleRef(oracle, c, dt=1e10)
        t0 = time.perf_counter()
        k = 0
        while k < nit and (k == 0 or time.perf_counter() - t0 < args.cpu_seconds):
            ref.step()
            k += 1
        per_it = (time.perf_counter() - t0) / k
        out["cpu_port_s_per_outer_it"] = round(per_it, 3)
        out["cpu_kind"] = (f"port (restated reference, sequential solvers, 1 core), first {k} "
                           f"outer iterations timed")
        out["gpu_fp64_over_cpu"] = round(per_it / (out["fp64"]["gpu_s"] / nit), 1)
    return out


def run_adjoint_c5(args):
    """The C5 configuration: sensitivity of the mean hot-wall Nusselt number
    to the hot-wall face temperatures of a natural-convection cavity (nx x nx
    quads, Ra = 1e5, hot faces at T_cold + (1 + N(0, 0.05)) K, seed 11) at the
    state the GPU loop reaches after c5_its outer iterations, with flow and
    densities frozen.  Adjoint: one forward and one adjoint solve give all
    the derivatives; checked against GPU central differences on 32 faces
    (seed 12).  J is affine in the continuous wall enthalpy of the frozen
    system, so no step adds truncation error, and a large one (c5_fd_step,
    default 10 K) keeps the differences far above the iterative solves'
    error: a 1 mK step leaves them at the 1e-2 level of that error, 0.1 K
    at 1e-4.  CPU: one solve of the same frozen system by the restated
    BiCGSTAB, times the 2 x faces solves of full differences."""
    import torch
    from fortranfvcell_gb300 import sensitivity as sv
    from fortranfvcell_gb300.cases import natural_convection_cavity
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    c = natural_convection_cavity(args.c5_nx, ra=1e5)
    cells, faces, _, _ = sv.wall_faces(c, 0.0)
    rng = np.random.default_rng(11)
    c["sedgeE"][cells, faces] = (c["t0"] - 0.5) + 1.0 + rng.normal(0.0, 0.05, cells.size)
    loop = SimpleLoop(c["coor"], c["ix"], c["nelcon"], c["num"], c["pedge"], c["sedge"], c["e"],
                      opts=simple_opts())
    loop.enable_energy(c["pedgeE"], c["sedgeE"], c["gravity"], c["t0"])
    t0 = time.perf_counter()
    res, _ = loop.iterate_energy(args.c5_its)
    loop_s = time.perf_counter() - t0
    sysd = sv.frozen_energy_system(c, loop)
    loop.close()
    prob = sv.NusseltProblem(c, sysd, tol=args.c5_tol)
    sv.nusselt_wall_gradient(prob, sysd["h_wall"])           # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    j, g = sv.nusselt_wall_gradient(prob, sysd["h_wall"])
    torch.cuda.synchronize()
    adj_s = time.perf_counter() - t0
    idx = np.random.default_rng(12).choice(g.size, min(32, g.size), replace=False)
    t0 = time.perf_counter()
    fd = sv.nusselt_fd(prob, sysd["h_wall"], idx, step=sysd["cp"] * args.c5_fd_step)
    torch.cuda.synchronize()
    fd_s = time.perf_counter() - t0
    prob_np = nusselt_numpy(prob)
    prob.close()
    rel = np.abs(g[idx] - fd) / np.maximum(np.abs(fd), 1e-300)
    out = {"workload": f"dJ/dT_wall, J = mean hot-wall Nu, natural convection {args.c5_nx}x"
                       f"{args.c5_nx} quads, Ra=1e5, {g.size} hot-wall faces, state after "
                       f"{args.c5_its} outer iterations (flow frozen)",
           "loop_s": round(loop_s, 3), "final_residuals": [float(f"{v:.3e}") for v in res[-1]],
           "J": round(j, 6), "adjoint_s": round(adj_s, 4),
           "fd_subset": {"faces": int(idx.size), "s": round(fd_s, 3),
                         "step_K": args.c5_fd_step, "solve_tol": args.c5_tol,
                         "max_rel_diff_vs_adjoint": float(f"{rel.max():.2e}")},
           "fd_all_faces_s_est": round(fd_s * g.size / idx.size, 3),
           "adjoint_over_fd_all": round(fd_s * g.size / idx.size / adj_s, 1),
           "dJ_dT_range": [float(f"{sysd['cp'] * g.min():.4e}"),
                           float(f"{sysd['cp'] * g.max():.4e}")]}
    if not args.no_cpu:
        from oracle import oracle
        n = c["numel"]
        ad = sysd["ad"].cpu().numpy()
        au = sysd["au"].cpu().numpy()
        b = sysd["b"].cpu().numpy()
        x = np.zeros(n)
        t0 = time.perf_counter()
        oracle.solver(ad, au.copy(), au.copy(), x, b.copy(), sysd["ia"], sysd["ja"], n,
                      sysd["nad"], True, 1e-12, 100000, 2, 1)
        cpu_solve = time.perf_counter() - t0
        out["cpu_port_one_solve_s"] = round(cpu_solve, 3)
        out["cpu_fd_all_faces_s_est"] = round(cpu_solve * 2 * g.size, 1)
        out["cpu_kind"] = ("port: restated sequential BiCGSTAB (1 core), one solve of the frozen "
                           "system, times 2 x faces for full central differences")
        # the same central differences through the restated reference solver
        # (pbicgstab_omp, Iterativos_omp.f:161-274, on all host threads).  Its
        # stopping test sqrt|b.z| < tol sqrt|d0| at the GPU differences'
        # tolerance left 1.0e-5 against the adjoint on one face of 32 (the
        # exit iteration alone sets that error: J is affine in h); a tenth
        # of it keeps the solves' error well below the 1e-5 bar
        threads = os.cpu_count() or 1
        tol_o = 0.1 * args.c5_tol
        t0 = time.perf_counter()
        fd_o = oracle_nusselt_fd(oracle, prob_np, idx, sysd["cp"] * args.c5_fd_step, tol_o,
                                 threads)
        fd_o_s = time.perf_counter() - t0
        rel_o = np.abs(g[idx] - fd_o) / np.maximum(np.abs(fd_o), 1e-300)
        rel_go = np.abs(fd - fd_o) / np.maximum(np.abs(fd_o), 1e-300)
        out["fd_subset"]["oracle"] = {
            "solver": f"restated pbicgstab_omp on {threads} threads, tol {tol_o:g}",
            "s": round(fd_o_s, 3), "max_rel_diff_vs_adjoint": float(f"{rel_o.max():.2e}"),
            "max_rel_diff_vs_gpu_fd": float(f"{rel_go.max():.2e}")}
    return out


def nusselt_numpy(prob):
    """The pieces of NusseltProblem as host arrays: J(h_w) = mean((h_w -
    h[rows]) / ca) * scale with A h = b_rest + sum_f ap_f h_f e_rows(f)."""
    s = prob.s
    return dict(ad=s["ad"].cpu().numpy(), au=s["au"].cpu().numpy(), ia=s["ia"], ja=s["ja"],
                nad=s["nad"], n=int(s["ad"].numel()), b_rest=prob.b_rest.cpu().numpy(),
                rows=s["rows"], ap=np.asarray(s["ap"]), ca=np.asarray(s["ca"]),
                scale=prob.scale, h_wall=np.asarray(s["h_wall"], np.float64))


def oracle_nusselt_fd(oracle, P, idx, step, tol, threads):
    """Central differences of J in the wall enthalpies idx, each J from one
    solve of the frozen enthalpy system by the restated reference BiCGSTAB
    (Solver.f dispatch: pbicgstab, or pbicgstab_omp with threads > 0)."""
    def jval(hw):
        b = P["b_rest"].copy()
        np.add.at(b, P["rows"], P["ap"] * hw)
        x = np.zeros(P["n"])
        st, _ = oracle.solver(P["ad"].copy(), P["au"].copy(), P["au"].copy(), x, b, P["ia"],
                              P["ja"], P["n"], P["nad"], True, tol, 100000, 2, 1,
                              omp_threads=threads)
        if st != 0:
            raise RuntimeError(f"restated BiCGSTAB status {st}")
        return float(np.mean((hw - x[P["rows"]]) / P["ca"]) * P["scale"])
    out = []
    for i in idx:
        e = np.zeros_like(P["h_wall"])
        e[i] = step
        out.append((jval(P["h_wall"] + e) - jval(P["h_wall"] - e)) / (2 * step))
    return np.array(out)


def c4_sides(ncases, seed=7):
    """Mesh sides of the batched workload: N = round(exp U[ln 32, ln 256])."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(32.0), np.log(256.0), ncases))).astype(int)


C4_WHICH = ((1, 2, "u"), (2, 2, "v"), (4, 2, "T"), (3, 1, "p'"))  # loop system, code, name


def c4_cases(ncases):
    """The C4 cases: N x N quads, N log-uniform in [32, 256] (seed 7), Re ~
    U[50, 400] (seed 8), a heated lid-driven cavity or a heated channel
    section by a seeded coin (seed 9), air, ideal gas with the energy
    equation."""
    from fortranfvcell_gb300.cases import heated_channel, heated_lid_cavity
    sides = c4_sides(ncases)
    res = np.random.default_rng(8).uniform(50.0, 400.0, ncases)
    kinds = np.where(np.random.default_rng(9).uniform(size=ncases) < 0.5, "cavity", "channel")
    cases = [(heated_channel if k == "channel" else heated_lid_cavity)(int(n), re=float(r))
             for n, r, k in zip(sides, res, kinds)]
    return sides, res, kinds, cases


def c4_loops(cases):
    from fortranfvcell_gb300.cells import SimpleLoop, simple_opts
    loops = []
    for c in cases:
        lp = SimpleLoop(c["coor"], c["ix"], c["nelcon"], c["num"], c["pedge"], c["sedge"],
                        c["e"], opts=simple_opts(matriz_u=1))
        lp.enable_energy(c["pedgeE"], c["sedgeE"], c["gravity"], c["t0"])
        loops.append(lp)
    return loops


C4_STAGES = (("u+v", (0, 1)), ("p'", (3,)), ("T", (2,)))   # SIMPLE order; C4_WHICH indices


def run_batched_c4(args):
    """The C4 configuration: ncases independent SIMPLE cases (c4_cases) of
    the ideal-gas loop with the energy equation, from rest, tolerances 1e-8.

    batch: the outer iterations of all cases together (fvc_simple_batch):
    each stage's solves of every case together (u and v, then p', then the
    enthalpy; one thread-block cluster per system, one launch per cluster
    size) with per-system convergence and masks, the cases' cell kernels
    side by side on 16 branches, one outer iteration of all cases one CUDA
    graph; two untimed outer iterations (the first captures the graph, the
    second captures it again with each system's iteration count as its
    weight), then c4_its timed, FP64 and mixed precision (FP32 iterations,
    FP64 refinement) from rest each.  sequential: one more outer iteration of
    every case alone (its own CUDA graph loop) after the FP64 batch.
    systems: the u, v, T, p' systems of the FP64 batch's last outer
    iteration, frozen, solved again per stage in one launch each -- on the
    reference's stopping tests, and FP64 against mixed on ||b - Ax|| <= 1e-8
    ||b|| for every system.  CPU: the restated iteration (the oracle's
    cells and sequential solvers, one core) on a seeded sample of cases,
    extrapolated by cells."""
    import torch
    from fortranfvcell_gb300 import Context, make_opts, pack_block_diagonal, mesh
    from fortranfvcell_gb300.cells import SimpleBatch
    t0 = time.time()
    sides, res_, kinds, cases = c4_cases(args.c4_cases)
    cells = int(sum(c["numel"] for c in cases))
    log(f"C4 setup: {len(cases)} cases, {cells} cells, {time.time() - t0:.1f} s")
    out = {"workload": f"{len(cases)} SIMPLE cases of air (ideal gas + energy), N x N quads, "
                       f"N = round(exp U[ln 32, ln 256]) seed 7 ({int(sides.min())}.."
                       f"{int(sides.max())}), Re ~ U[50, 400] seed 8, "
                       f"{int((kinds == 'cavity').sum())} heated lid-driven cavities and "
                       f"{int((kinds == 'channel').sum())} heated channel sections (seed 9), "
                       f"{cells} cells in all, from rest, solver tolerances 1e-8",
           "batch": {}}
    nit = args.c4_its
    fp64_loops = None
    # precision of the p' solves, and of the u, v and enthalpy solves: FP64;
    # mixed p' (the C3 default: the enthalpy's FP32 sweeps can stall, and a
    # batch does not finish a stalled solve in FP64); mixed everywhere
    for name, prec, prec_u in (("fp64", "fp64", "fp64"), ("mixed", "mixed", "fp64"),
                               ("mixed_all", "mixed", "mixed")):
        loops = c4_loops(cases)
        bt = SimpleBatch(loops, prec, prec_u)
        try:
            bt.iterate(2, 4)                 # captures, then captures with the shares
            torch.cuda.synchronize()
            l0 = _kernel_launches()
            t1 = time.perf_counter()
            res, its = bt.iterate(nit, 4)
            el = time.perf_counter() - t1
            launches = _kernel_launches() - l0
        except Exception as e:  # a stalled mixed BiCGSTAB ends the call (FVC_ERR_NOCONV)
            out["batch"][name] = {"precision": [prec, prec_u], "error": str(e)}
            bt.close()
            for lp in loops:
                lp.close()
            continue
        bt.close()
        last = its[-1]
        out["batch"][name] = {"precision_pc_u": [prec, prec_u],
            "outer_its": nit, "s": round(el, 3), "s_per_outer_it": round(el / nit, 4),
            "case_outer_its_per_s": round(len(cases) * nit / el, 1),
            "cell_outer_its_per_s": round(cells * nit / el, 1),
            "gpu_launches_per_outer_it": int(launches / nit),
            "solver_iterations_last": {n: {"median": int(np.median(last[:, k])),
                                           "max": int(last[:, k].max())}
                                       for k, n in enumerate(("u", "v", "p'", "T"))},
            "residual_last_max": [float(f"{v:.3e}") for v in res[-1].max(axis=0)]}
        log(f"C4 batch {name}: {el / nit * 1e3:.1f} ms per outer iteration of all cases")
        if name == "fp64":
            fp64_loops = loops
        else:
            for lp in loops:
                lp.close()
    for name in ("mixed", "mixed_all"):
        if "s" in out["batch"].get(name, {}):
            out["batch"][name]["over_fp64"] = round(out["batch"]["fp64"]["s"]
                                                    / out["batch"][name]["s"], 3)
    # the next outer iteration of every FP64 case alone, each its own graph
    for lp in fp64_loops:
        lp.use_graph(True)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for lp in fp64_loops:
        lp.iterate_energy(1)
    torch.cuda.synchronize()
    seq = time.perf_counter() - t1
    out["sequential"] = {"s_per_outer_it": round(seq, 4),
                         "note": "every case's next outer iteration alone, its own CUDA graph "
                                 "(the first run of each case's graph includes its capture)"}
    out["batch_over_sequential"] = round(seq / out["batch"]["fp64"]["s_per_outer_it"], 2)
    # the systems of that outer iteration, frozen, per stage in one launch each
    systems, codes = [], []
    for c, lp in zip(cases, fp64_loops):
        ia, ja, nad = mesh.datastruc(c["ident"], 1, True)
        for which, code, _ in C4_WHICH:
            ad, au, b = lp.system(which)
            systems.append(dict(ad=ad, au=au, ia=ia, ja=ja, n=ad.size, nad=nad, b=b))
            codes.append(code)
    for lp in fp64_loops:
        lp.close()
    codes = np.array(codes, np.int32)
    stream = torch.cuda.Stream()
    nw = len(C4_WHICH)

    def batch_of(idx):
        sub = [systems[i] for i in idx]
        pk = pack_block_diagonal(sub)
        c = Context(device=0, stream=stream)
        c.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                     pk["ja"])
        bv = np.zeros(pk["neq"])
        for sy, r in zip(sub, pk["rows"]):
            bv[r] = sy["b"]
        return dict(ctx=c, pk=pk, bd=torch.from_numpy(bv).cuda(),
                    xd=torch.zeros(pk["neq"], dtype=torch.float64, device="cuda"),
                    codes=codes[idx], idx=np.array(idx))

    def run(bt, opts, reps=2):
        with torch.cuda.stream(stream):
            kw = dict(codes=bt["codes"], raise_on_error=False)
            bt["ctx"].solve_batched(bt["pk"]["row_start"], bt["bd"], bt["xd"], C4_TOL, 50000,
                                    opts, **kw)
            r = [bt["ctx"].solve_batched(bt["pk"]["row_start"], bt["bd"], bt["xd"], C4_TOL,
                                         50000, opts, **kw) for _ in range(reps)]
        rc, st = min(r, key=lambda q: q[1][0].solve_ms)
        return dict(ms=st[0].solve_ms, rc=int(rc), st=st)

    stages = [(name, batch_of([i for i in range(len(systems)) if i % nw in fl]))
              for name, fl in C4_STAGES]
    sysout = {"systems": len(systems), "rows": int(sum(sy["n"] for sy in systems))}
    per, tot = {}, 0.0
    for name, bt in stages:
        r = run(bt, make_opts("fp64", init=1))
        per[name] = round(r["ms"], 3)
        tot += r["ms"]
    sysout["reference_tests"] = {"per_stage_ms": per, "total_ms": round(tot, 3)}
    rule = {}
    # the automatic form (one thread-block cluster per system, sized to it,
    # one launch per size), and both precisions as groups of blocks sharing
    # one cooperative launch
    variants = (("fp64", "fp64", 0), ("mixed", "mixed", 0), ("fp64_groups", "fp64", 1),
                ("mixed_groups", "mixed", 1))
    for key, prec, csize in variants:
        o = make_opts(prec, init=1, stop_rule=1, cluster_size=csize)
        per, tot, wr, ok, fin = {}, 0.0, 0.0, True, 0
        for name, bt in stages:
            r = run(bt, o)
            per[name] = round(r["ms"], 3)
            tot += r["ms"]
            wr = max(wr, max(t.rel_residual for t in r["st"]))
            ok = ok and r["rc"] == 0
            if prec == "mixed":
                fin += sum(1 for t in r["st"] if t.iterations > t.inner_iterations)
        rule[key] = dict(per_stage_ms=per, total_ms=round(tot, 3),
                         worst_rel_residual=float(f"{wr:.3e}"), all_converged=ok,
                         form="groups" if csize == 1 else "clusters sized per system")
        if prec == "mixed":
            rule[key]["fp64_finished_systems"] = fin
    sysout["relres_rule"] = dict(rule="||b - Ax|| <= 1e-8 ||b|| for every system, per stage",
                                 **rule,
                                 mixed_over_fp64=round(rule["fp64"]["total_ms"]
                                                       / rule["mixed"]["total_ms"], 2),
                                 mixed_over_fp64_groups=round(rule["fp64_groups"]["total_ms"]
                                                              / rule["mixed"]["total_ms"], 2))
    for _, bt in stages:
        bt["ctx"].close()
    out["systems_of_one_outer_iteration"] = sysout
    if not args.no_cpu:
        from oracle import oracle
        from oracle.simple_ref import GasSimpleRef
        order = np.random.default_rng(3).permutation(len(cases))
        done_cells, el = 0, 0.0
        for k in order:
            ref = GasSimpleRef(oracle, cases[k], dt=1e10, matriz_u=1)
            t1 = time.perf_counter()
            ref.step()
            el += time.perf_counter() - t1
            done_cells += cases[k]["numel"]
            if el > args.cpu_seconds:
                break
        cpu_it = el * cells / done_cells
        out["cpu_port_s_per_outer_it"] = round(cpu_it, 3)
        out["cpu_kind"] = (f"port: the restated iteration (oracle cells and sequential solvers, "
                           f"1 core), the first outer iteration of a seeded sample of cases "
                           f"({done_cells} cells, {el:.1f} s), extrapolated by cells")
        out["batch_over_cpu"] = round(cpu_it / out["batch"]["fp64"]["s_per_outer_it"], 1)
    return out


def _kernel_launches():
    import fortranfvcell_gb300 as fvc
    return fvc.kernel_launches()


C2_MESHES = (("1M", (("quad", 1024), ("tri", 724), ("mixed", 836))),
             ("4M", (("quad", 2048), ("tri", 1448), ("mixed", 1672))))


def unsymmetric_variant(ad, au, ia, n, seed=5, skew=0.4):
    """A convection-like unsymmetric M-matrix on a CSRD p' structure: each
    off-diagonal scaled by 1 + skew U[-1, 1], the diagonal the row's
    absolute off-diagonal sum plus 5% (plus 1e-3): diagonally dominant."""
    rng = np.random.default_rng(seed)
    au2 = au * (1.0 + skew * rng.uniform(-1.0, 1.0, au.size))
    rows = np.repeat(np.arange(n), np.diff(ia))
    ad2 = np.bincount(rows, weights=np.abs(au2), minlength=n) * 1.05 + 1e-3
    return ad2, au2


def run_c2(args):
    """The C2 configuration: standalone SpMV and PCG / BiCGSTAB on p'
    systems of jittered (+-20%, seed 1234) unit-square meshes of about 1M
    and 4M cells: quadrilaterals, triangles (every quad cut along a seeded
    diagonal) and the 50/50 mixed mesh; RCM; CSRD (matriz 1) and, for the
    one-type meshes, ELLPACK (matriz 4, the reference's width-3/4 ELL);
    b ~ U[-1, 1] seed 42, x0 = 0, ||b - Ax|| <= 1e-8 ||b||.  Per leg: the
    FP64 and the mixed PCG (solves/s, us per iteration), the FP64 FMA and
    FP32 SpMV (GB/s on true nonzeros), and the CPU port's pcg_omp per
    iteration on all host threads times the FP64 iteration count.
    BiCGSTAB legs: an unsymmetric variant of the mixed-mesh structure.
    1M-cell working sets fit in L2 (129 MB) across iterations: those legs
    are labelled L2-resident; the 4M ones exceed it."""
    import torch
    from fortranfvcell_gb300 import Context, make_opts, mesh
    from oracle import oracle
    threads = os.cpu_count() or 1
    stream = torch.cuda.Stream()
    hbm, _ = peaks()
    legs = []

    def timed_solve(ctx, code, bd, xd, opts):
        with torch.cuda.stream(stream):
            ctx.solve(code, bd, xd, TOL, 200000, opts)      # warm-up
            st = ctx.solve(code, bd, xd, TOL, 200000, opts)
        return st

    def spmv_gbs(ctx, bd, nnz, n):
        y = torch.empty_like(bd)
        x32, y32 = bd.float(), torch.empty(n, dtype=torch.float32, device="cuda")
        res = {}
        for name, fn, nbytes in (("fp64_fma", lambda: ctx.spmv_fast(bd, y), 12 * nnz + 24 * n),
                                 ("fp32", lambda: ctx.spmv_f32(x32, y32), 6 * nnz + 12 * n)):
            with torch.cuda.stream(stream):
                for _ in range(3):
                    fn()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(20):
                    fn()
                e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 20
            gbs = nbytes / (ms * 1e-3) / 1e9
            res[name] = {"gbs": round(gbs, 1), "frac_of_peak": round(gbs / hbm, 3)}
        return res

    for size, kinds in C2_MESHES:
        for kind, nx in kinds:
            m = mesh.square_mesh(nx, kind=kind, jitter=0.2, seed=1234)
            for matriz in ((1, 4) if kind != "mixed" else (1,)):
                sy = mesh.pressure_system(m, matriz=matriz, unsym=True, pin_cell=1)
                n = sy.neq
                b = np.random.default_rng(42).uniform(-1.0, 1.0, n)
                ctx = Context(device=0, stream=stream)
                ctx.set_matrix(matriz, True, n, sy.nad, sy.ad, sy.au, sy.au, sy.ia, sy.ja)
                nnz = ctx.info()["nnz_off"]
                bd = torch.from_numpy(b).cuda()
                xd = torch.zeros(n, dtype=torch.float64, device="cuda")
                leg = {"cells": n, "mesh": kind, "format": "CSRD" if matriz == 1 else "ELLPACK",
                       "solver": "PCG", "nnz_off": nnz,
                       "l2": "L2-resident across iterations (working set < 129 MB)"
                             if size == "1M" else "exceeds L2"}
                for prec in ("fp64", "mixed"):
                    st = timed_solve(ctx, 1, bd, xd, make_opts(prec, init=1, stop_rule=1,
                                                               refine_tol=TOL))
                    its = st.iterations if prec == "fp64" else st.inner_iterations
                    leg[prec] = {"solves_per_s": round(1000.0 / st.solve_ms, 3),
                                 "iterations": int(its),
                                 "us_per_iteration": round(st.solve_ms * 1e3 / max(its, 1), 2)}
                leg["mixed_over_fp64"] = round(leg["mixed"]["solves_per_s"]
                                               / leg["fp64"]["solves_per_s"], 3)
                leg["spmv"] = spmv_gbs(ctx, bd, nnz, n)
                ctx.close()
                if not args.no_cpu:
                    per = oracle_s_per_iteration(sy.ad, sy.au, sy.ia, sy.ja, n, sy.nad, b,
                                                 threads, 3, matriz)
                    k = int(max(3, min(500, 1.0 / max(per, 1e-6))))
                    xo = np.zeros(n)
                    t0 = time.perf_counter()
                    oracle.pcg_omp_sample(sy.ad, sy.au, xo, b.copy(), sy.ia, sy.ja, n, sy.nad,
                                          1e-300, k, matriz, threads)
                    per = (time.perf_counter() - t0) / k
                    leg["cpu_port"] = {"solves_per_s": round(1.0 / (per * leg["fp64"]["iterations"]),
                                                             5),
                                       "ms_per_iteration": round(per * 1e3, 3),
                                       "sample": f"{k} pcg_omp iterations on {threads} threads x "
                                                 f"the FP64 iteration count"}
                legs.append(leg)
                log(f"C2 {size} {kind} matriz {matriz}: fp64 {leg['fp64']['solves_per_s']} "
                    f"mixed {leg['mixed']['solves_per_s']} solves/s")
            if kind == "mixed":     # BiCGSTAB on an unsymmetric system of the same structure
                sy = mesh.pressure_system(m, matriz=1, unsym=True, pin_cell=1)
                n = sy.neq
                ad2, au2 = unsymmetric_variant(sy.ad, sy.au[:sy.nad], sy.ia, n)
                b = np.random.default_rng(42).uniform(-1.0, 1.0, n)
                ctx = Context(device=0, stream=stream)
                ctx.set_matrix(1, True, n, sy.nad, ad2, au2, au2, sy.ia, sy.ja)
                bd = torch.from_numpy(b).cuda()
                xd = torch.zeros(n, dtype=torch.float64, device="cuda")
                leg = {"cells": n, "mesh": kind, "format": "CSRD", "solver": "BiCGSTAB",
                       "matrix": "p' structure, off-diagonals x (1 + 0.4 U[-1,1]) seed 5, "
                                 "diagonal 1.05 x |row| + 1e-3",
                       "l2": "L2-resident across iterations (working set < 129 MB)"
                             if size == "1M" else "exceeds L2"}
                for prec in ("fp64", "mixed"):
                    st = timed_solve(ctx, 2, bd, xd, make_opts(prec, init=1, stop_rule=1,
                                                               refine_tol=TOL))
                    its = st.iterations if prec == "fp64" else st.inner_iterations
                    leg[prec] = {"solves_per_s": round(1000.0 / st.solve_ms, 3),
                                 "iterations": int(its),
                                 "us_per_iteration": round(st.solve_ms * 1e3 / max(its, 1), 2)}
                leg["mixed_over_fp64"] = round(leg["mixed"]["solves_per_s"]
                                               / leg["fp64"]["solves_per_s"], 3)
                ctx.close()
                if not args.no_cpu:
                    xo = np.zeros(n)
                    t0 = time.perf_counter()
                    rc, so = oracle.solver(ad2, au2.copy(), au2.copy(), xo, b.copy(), sy.ia,
                                           sy.ja, n, sy.nad, True, TOL, 100000, 2, 1,
                                           omp_threads=threads)
                    el = time.perf_counter() - t0
                    leg["cpu_port"] = {"solves_per_s": round(1.0 / el, 4),
                                       "iterations": int(so.iterations),
                                       "sample": f"one whole pbicgstab_omp solve on {threads} "
                                                 f"threads (the reference's stopping test)"}
                legs.append(leg)
    return {"workload": "p' systems of jittered unit-square meshes (seed 1234), ~1M and ~4M "
                        "cells, quad / tri / mixed, CSRD and ELLPACK, RCM, b~U[-1,1] seed 42, "
                        "x0 = 0, ||b-Ax|| <= 1e-8 ||b||; BiCGSTAB on an unsymmetric variant",
            "legs": legs}


def run_profile_case(args):
    """Profiling case for ncu: the bench workload, each solver run once for
    a fixed number of iterations (no convergence wait), plus one SpMV."""
    import torch
    from fortranfvcell_gb300 import Context, make_opts
    s, b = build_system_gpu(args.nx)
    n = s.neq
    ctx = Context()
    ctx.set_matrix(1, True, n, s.nad, s.ad, s.au, s.au, s.ia, s.ja)
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros(n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(bd)
    torch.cuda.synchronize()
    ctx.spmv_fast(bd, y)
    ctx.spmv(bd, y)
    # one short solve of each kind first: the timed ones exclude module loading
    ctx.solve(1, bd, xd, 1e-30, 5, make_opts("mixed", init=1), raise_on_error=False)
    ctx.solve(1, bd, xd, 1e-30, 5, make_opts("fp64", init=1, stop_rule=1), raise_on_error=False)
    out = {}
    for name, opts in (("mixed", make_opts("mixed", init=1)),
                       ("fp64", make_opts("fp64", init=1, stop_rule=1))):
        st = ctx.solve(1, bd, xd, 1e-30, args.profile_its, opts, raise_on_error=False)
        out[name] = {"iterations": st.iterations, "ms": round(st.solve_ms, 3),
                     "us_per_iteration": round(st.solve_ms * 1e3 / max(st.iterations, 1), 2)}
    # the FP32 operator the mixed solves built, three times
    x32 = bd.float()
    y32 = torch.empty_like(x32)
    for _ in range(3):
        ctx.spmv_f32(x32, y32)
    torch.cuda.synchronize()
    out["cells"] = n
    out["nnz_off"] = ctx.info()["nnz_off"]
    return out


def run_reference(args):
    """The CPU restatement of the reference's OpenMP path (pcg_omp with
    matvec_csrd_omp and dot_ompL4, Iterativos_omp.f:30-127), all host
    threads, same workload and setup chain (the restated Adjacency.f,
    Reord.f, Numeq.f, Datastruct.f and the p' assembly).  One whole solve
    from x = 0 on the GPU arm's rule ||r|| <= 1e-8 ||b|| gives the
    iteration count and its own time; each step then times a bounded
    sample of the reference's loop, and solves/s = 1 / (s per iteration x
    that count).  A 1-thread sample is reported beside it."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    from oracle import oracle
    t0 = time.time()
    m = build_mesh(args.nx)
    nelcon = oracle.adjacency_mixed(m.ix, m.nnode, m.nshared)
    num = oracle.reord(nelcon)
    ident = oracle.numeq(num, nelcon)
    ia, ja, nad = oracle.datastruc(ident, 1, True)
    ad, au = oracle.pform_pressure(m.coor, m.ix, m.nshared, nelcon, num, ia, ja, 1, True,
                                   pin_cell=1)
    n = m.numel
    b = np.random.default_rng(42).uniform(-1.0, 1.0, n)
    log(f"reference setup {time.time() - t0:.1f} s")
    threads = os.cpu_count() or 1
    _, its, whole_s, rel, rc = oracle_whole_solve(ad, au, ia, ja, n, nad, b, threads)
    log(f"reference whole solve: {its} iterations, {whole_s:.1f} s, relres {rel:.3e}")
    sample_its = args.ref_sample_its
    times = []
    for k in range(args.warmup + args.steps):
        per = oracle_s_per_iteration(ad, au, ia, ja, n, nad, b, threads, sample_its)
        if k >= args.warmup:
            times.append(per * sample_its)
    per_it = statistics.mean(times) / sample_its
    value = 1.0 / (per_it * its)
    per1 = oracle_s_per_iteration(ad, au, ia, ja, n, nad, b, 1, 3)
    k1 = int(max(3, min(2000, 3.0 / max(per1, 1e-6))))
    per1 = oracle_s_per_iteration(ad, au, ia, ja, n, nad, b, 1, k1)
    return {
        "metric": "PCG solves/s to ||b-Ax||/||b||<=1e-8, p' system, mixed FP32/FP64 "
                  "(plain FP64 and SpMV GB/s alongside)",
        "value": round(value, 6), "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(times) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": f"p' Jacobi-PCG, jittered mixed tri/quad unit square, {n} cells "
                               f"(nx={args.nx}), RCM, CSRD, b~U[-1,1] seed 42, x0=0",
                   "cells": n, "tol_rel_residual": TOL},
        "cpu_baseline": {"value": round(value, 6), "unit": "solves/s", "cores": threads,
                         "kind": "port",
                         "sample": f"each step {sample_its} pcg_omp iterations on {threads} "
                                   f"threads; solves/s = 1/(s per iteration x {its}), the "
                                   f"iterations of one whole solve to ||r|| <= {TOL:g} ||b||",
                         "whole_solve": {"iterations": its, "s": round(whole_s, 3),
                                         "solves_per_s": round(1.0 / whole_s, 6),
                                         "rel_residual_fp64": float(f"{rel:.3e}"),
                                         "status": rc},
                         "one_thread": {"value": round(1.0 / (per1 * its), 6),
                                        "unit": "solves/s", "cores": 1,
                                        "sample": f"{k1} pcg_omp iterations on 1 thread "
                                                  f"({per1 * 1e3:.2f} ms each) x {its}"},
                         "build": "gcc -O3 -fopenmp -ffp-contract=off (oracle/Makefile)"},
        "e2e": {"value": round(value, 6), "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_c4_profile_case(args):
    """One frozen C4 stage solved twice, the second solve inside a profiler
    range: the workload of the C4 stage profiles."""
    import torch
    from fortranfvcell_gb300 import Context, make_opts, pack_block_diagonal, mesh
    from fortranfvcell_gb300.cells import SimpleBatch
    stage, prec, csize = args.c4_profile.split(":")
    which, code = {"p": (3, 1), "T": (4, 2)}[stage]
    _, _, _, cases = c4_cases(args.c4_cases)
    loops = c4_loops(cases)
    bt = SimpleBatch(loops, "fp64")
    bt.iterate(3, 4)
    bt.close()
    systems = []
    for c, lp in zip(cases, loops):
        ia, ja, nad = mesh.datastruc(c["ident"], 1, True)
        ad, au, b = lp.system(which)
        systems.append(dict(ad=ad, au=au, ia=ia, ja=ja, n=ad.size, nad=nad, b=b))
    for lp in loops:
        lp.close()
    pk = pack_block_diagonal(systems)
    ctx = Context(device=0)
    ctx.set_matrix(1, True, pk["neq"], pk["nad"], pk["ad"], pk["au"], pk["au"], pk["ia"],
                   pk["ja"])
    bv = np.zeros(pk["neq"])
    for sy, r in zip(systems, pk["rows"]):
        bv[r] = sy["b"]
    bd = torch.from_numpy(bv).cuda()
    xd = torch.zeros(pk["neq"], dtype=torch.float64, device="cuda")
    o = make_opts(prec, init=1, stop_rule=1, cluster_size=int(csize))
    codes = np.full(len(systems), code, np.int32)
    out = {"stage": stage, "precision": prec, "cluster_size": int(csize),
           "systems": len(systems), "rows": int(pk["neq"])}
    for rep in range(2):
        if rep == 1:
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
        rc, st = ctx.solve_batched(pk["row_start"], bd, xd, C4_TOL, 50000, o,
                                   raise_on_error=False, codes=codes)
        if rep == 1:
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()
        out[f"solve{rep}"] = {"status": int(rc), "ms": round(st[0].solve_ms, 3),
                              "iterations": int(sum(t.iterations for t in st))}
    ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=NX_DEFAULT)
    ap.add_argument("--inner-tol", type=float, default=0.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-simple", action="store_true", help="skip the C1 SIMPLE leg")
    ap.add_argument("--no-c2", action="store_true",
                    help="skip the C2 legs (1M / 4M, quad / tri / mixed, CSRD / ELL, PCG / "
                         "BiCGSTAB)")
    ap.add_argument("--simple-nx", type=int, default=64)
    ap.add_argument("--simple-its", type=int, default=200)
    ap.add_argument("--c3-nx", type=int, default=512,
                    help="natural-convection C3 leg: cells per side (0 skips it)")
    ap.add_argument("--c3-ra", type=float, default=1.0e6)
    ap.add_argument("--c3-its", type=int, default=30)
    ap.add_argument("--c3-precision-u", default="fp64", choices=["fp64", "mixed"],
                    help="natural-convection C3 leg: precision of the momentum and enthalpy "
                         "solves in its mixed run")
    ap.add_argument("--c5-nx", type=int, default=256,
                    help="adjoint C5 leg: cells per side (0 skips it)")
    ap.add_argument("--c5-its", type=int, default=200)
    ap.add_argument("--c5-fd-step", type=float, default=10.0,
                    help="adjoint C5 leg: central-difference step of the wall temperatures (K)")
    ap.add_argument("--c5-tol", type=float, default=1e-12,
                    help="adjoint C5 leg: relative tolerance of the forward and adjoint solves")
    ap.add_argument("--c4-cases", type=int, default=256,
                    help="batched C4 leg: number of cases (0 skips it)")
    ap.add_argument("--c4-its", type=int, default=5,
                    help="batched C4 leg: timed outer iterations of all cases")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="bound on the CPU samples of the configuration legs")
    ap.add_argument("--ref-sample-its", type=int, default=300)
    ap.add_argument("--profile-leg", choices=["c1", "c2", "c3", "c4", "c5"], default=None,
                    help="profiling: run only this leg (no CPU side) and print its JSON")
    ap.add_argument("--profile-its", type=int, default=0,
                    help="profiling case: run each solver once for this many iterations")
    ap.add_argument("--c4-profile", default=None, metavar="STAGE:PREC:CLUSTER",
                    help="profiling case: one C4 stage (p or T) of --c4-cases cases, frozen "
                         "after 3 FP64 batch outer iterations, solved twice to ||r|| <= 1e-8 "
                         "||b|| in precision PREC (fp64 / mixed) with fvc_opts.cluster_size "
                         "CLUSTER; the second solve between cudaProfilerStart and Stop (for "
                         "ncu --profile-from-start off)")
    args = ap.parse_args()
    if args.profile_its > 0:
        print(json.dumps(run_profile_case(args)), flush=True)
        return
    if args.c4_profile:
        print(json.dumps(run_c4_profile_case(args)), flush=True)
        return
    if args.profile_leg:
        args.no_cpu = True
        leg = {"c1": run_simple_c1, "c2": run_c2, "c3": run_gas_c3, "c4": run_batched_c4,
               "c5": run_adjoint_c5}[args.profile_leg]
        print(json.dumps(leg(args)), flush=True)
        return
    if args.warmup < 3:
        log("note: the timing rules want >= 3 warm-up steps")
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
