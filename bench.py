#!/usr/bin/env python
"""Benchmark: SEMO's outer iteration (momentum + pressure correction) on one GB300.

Workload: jittered hex box 128^3 (2,097,152 cells, 6,340,608 faces), two-phase
VOF fields (water drop in air, gravity) with seeded old and second-old
velocities, seeded synthetic inputs.  One step is one outer iteration of the
pressure-based solver with one pressure correction:
  momentum  cell viscosity, face values, stencil min/max, five LSQ gradients,
            BDF2 + convection + diffusion assembly (one matrix, three RHS), the
            three solves (BiCGStab, Jacobi) to 1e-9, U/V/W update;
  pressure  EOS and face values, gravity source, stencil pass, face-loop
            assembly, smoothed-aggregation AMG setup, CG to a 1e-8 FP64
            relative residual, two Gauss-Green sweeps, P/U/V/W update.
Successive steps continue from the updated fields, as SEMO's outer loop does.
Mesh data (several GB) is far larger than the 129 MB L2, so no flush is
needed between steps.

  value          Mcells/s per outer iteration, inputs resident in HBM, FP32 AMG
                 inside FP64 CG for the pressure
  pressure_pass  the pressure-correction pass alone (calcPressureEq)
  e2e            the outer iteration through the public C-ABI with host buffers:
                 fields and old velocities copied in, the iteration, fields
                 copied out, every step (wall clock)
  fp64           the same with an all-FP64 hierarchy and V-cycle
  adjoint        A^T lambda = dJ/dx on the forward hierarchy, time vs the forward solve
  coupled        calcCompCoupledEq (ideal gas, 5x5 blocks) on 6 x 96^3 tetrahedra,
                 FP64 and mixed
  large          the 256^3 case: outer iterations, the adjoint transpose solve on
                 the same hierarchy, per-kernel HBM fractions, device memory
  roofline       the dominant single-launch kernel (HBM and FP64 fractions), the
                 two SpMVs timed alone and a whole CG iteration
  error_vs_oracle  the GPU path against the FP64 CPU oracle on this workload
                 (systems, solutions, fields after one outer iteration)

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 128]
"""
from __future__ import annotations

import argparse
import atexit
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcells/s per outer iter to 1e-8 rel. residual: FP32-mixed vs FP64 GPU; adj/fwd"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "dram_traffic.json")
UNIT = "Mcells/s"


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region.

    Started before the warm-up (its start-up initialises NVML, which must not
    fall inside the timed loop); `wait_first()` blocks until it has sampled
    once, `mark(t0, t1)` records the timed window, and `summary()` keeps the
    samples taken inside it (all of them if the window was shorter than the
    sampling period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.window = None
        self.t_start = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            atexit.register(self.stop)
        except OSError:
            self.proc = None
        self.t_start = time.monotonic()
        return self

    def __enter__(self):
        return self.start()

    def settle(self, seconds: float = 3.0) -> None:
        """Wait until `seconds` after the sampler started.  Measured on a GB300:
        an outer iteration that ran 1-1.3 s after nvidia-smi started took
        75 ms instead of 22 ms (once; later ones were unaffected), so the
        sampler starts before the case is built and the timing waits for this."""
        if self.t_start is not None:
            rest = self.t_start + seconds - time.monotonic()
            if rest > 0:
                time.sleep(rest)

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([time.monotonic()] + [x.strip() for x in line.split(",")])

    def wait_first(self, timeout: float = 10.0) -> None:
        t_end = time.monotonic() + timeout
        while self.proc and not self.rows and time.monotonic() < t_end:
            time.sleep(0.02)

    def mark(self, t0: float, t1: float) -> None:
        self.window = (t0, t1)

    def stop(self) -> None:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.proc = None

    def __exit__(self, *exc):
        self.stop()

    def summary(self) -> dict:
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        rows = self.rows
        if self.window:
            inside = [r for r in rows if self.window[0] <= r[0] <= self.window[1]]
            rows = inside if inside else rows
        rows = [r[1:] for r in rows]
        sm = [v for v in (num(r[1]) for r in rows if len(r) > 2) if v is not None]
        mx = [v for v in (num(r[2]) for r in rows if len(r) > 2) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({nm for r in rows for k, nm in enumerate(names)
                          if len(r) > 5 + k and r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def hbm_peak() -> tuple:
    if os.path.exists(PEAKS):
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stencil_algo_bytes(m: dict) -> float:
    """Compulsory bytes of one full k_stencil launch, the survey's formula.

    LSQ gradients of k = 5 fields: N (24 centroid + 48 M^-1 + 4 row pointer
    + 8k phi + 24k grad phi) + 4 nnz_s = 236 B a cell + 4 B a stencil entry;
    the stencil min/max of the same 5 fields reads nothing more and writes
    10 planes (80 B a cell).
    """
    return m["cells"] * (236 + 80) + 4 * m["stencil_nnz"]


def stencil_design_bytes(m: dict) -> float:
    """Bytes this design's k_stencil moves when each array is touched once.

    per cell: P,U,V,W,VF (40) + stencil row pointer (4) + M^-1 (48) + the
    weight sums (24) read, 15 gradient components (120) + 10 min/max (80)
    written; per stencil entry: cell index (4) + precomputed LSQ weight vector
    w*d (24); per boundary face: weight vector (24) + 5 face values (40).
    The weight vectors trade bytes for FP64 operations.
    """
    return (m["cells"] * (40 + 4 + 48 + 24 + 120 + 80) + m["stencil_nnz"] * (4 + 24)
            + m["boundary_faces"] * (24 + 40))


def stencil_fp64_flops(m: dict) -> float:
    """FP64 flops of one full k_stencil launch (an FMA counts 2).

    per stencil entry and per boundary face 15 FMAs (3 components x 5
    fields); per cell 15 FMAs (phi_i times the weight sums) + 45 FMAs
    (M^-1 applied to 5 vectors).
    """
    return 2.0 * (15 * (m["stencil_nnz"] + m["boundary_faces"]) + 60 * m["cells"])


def spmv_algo_bytes(n: int, nnz: int, value_bytes: int) -> float:
    """Compulsory bytes of y = A x, CSR (survey formula): FP64 12 nnz + 4(N+1)
    + 16N; FP32 values and vectors 8 nnz + 4(N+1) + 8N."""
    return (4 + value_bytes) * nnz + 4 * (n + 1) + 2 * value_bytes * n


def pcg_iteration_bytes(levels: list) -> float:
    """Compulsory bytes of one preconditioned CG iteration (V(2,2) cycle,
    Chebyshev degree 2), each array counted once per kernel that touches it.

    per level above the coarsest (values and vectors of `value_bytes` V):
      4 operator sweeps (pre-smoothing, residual, two post-smoothing steps),
      each as an SpMV, plus the D^-1 and b reads of the smoothing sweeps (3 x 2Vn);
      restriction y = R r and prolongation x += P x_c as SpMVs (+ Vn for the
      read-modify-write of x);
    coarsest level: its dense FP64 inverse (8 n^2) and two vectors;
    finest level, FP64: the outer SpMV (12 nnz + 4(N+1) + 16N), the update
      of p (16N), the dot products' reads of r and q (16N) and the x, r update
      (x and r read and written, p and q read: 48N) plus the FP32 copy of r (VN).
    """
    total = 0.0
    for l, L in enumerate(levels):
        n, V = L["rows"], L["value_bytes"]
        if L["layout"] < 0:   # coarsest: dense inverse
            total += 8.0 * n * n + 2 * V * n
            continue
        nc = levels[l + 1]["rows"]
        total += 4 * spmv_algo_bytes(n, L["nnz_A"], V) + 3 * 2 * V * n
        total += (4 + V) * L["nnz_R"] + 4 * (nc + 1) + V * n + V * nc
        total += (4 + V) * L["nnz_P"] + 4 * (n + 1) + V * nc + 2 * V * n
    L0 = levels[0]
    N = L0["rows"]
    total += spmv_algo_bytes(N, L0["nnz_A"], 8) + 16 * N + 16 * N + 48 * N + L0["value_bytes"] * N
    return total


def pface_algo_bytes(m: dict) -> float:
    """Compulsory bytes of one k_pface launch, the survey's formula: per
    internal face 136 B (owner/neighbour 8, 13 geometry doubles 104, two
    off-diagonals 16, UnF 8), per cell 264 B (31 gathered doubles + diagonal
    and right-hand side)."""
    return m["internal_faces"] * 136 + m["cells"] * 264


def pface_bytes(m: dict) -> float:
    """Bytes this design's k_pface moves (each array touched once).

    per internal face: owner/neighbour (8), normal, e_PN, skew (72), alpha (8),
    4 face constants (32), 2 CSR slots (8) read; 2 off-diagonals (16) and coef,
    flux, UnF (24) written; per cell, read once: 1/rho, P, U, V, W, 12 gradient
    components, 6 min/max, 3 gravity sources (216).
    """
    return m["internal_faces"] * (8 + 72 + 8 + 32 + 8 + 16 + 24) + m["cells"] * 216


def mface_bytes(m: dict) -> float:
    """Bytes this design's k_mface moves (each array touched once).

    per internal face: as k_pface's face reads (128) plus 8 face terms (64)
    and 2 off-diagonals (16) written; per cell, read once: 1/rho, rho, 1/mu,
    P, U, V, W, 15 gradient components, 8 limits, 3 gravity sources (264).
    """
    return m["internal_faces"] * (8 + 72 + 8 + 32 + 8 + 64 + 16) + m["cells"] * 264


# stage -> (kernel, algorithmic bytes, design bytes) per launch; each of these
# stages is one launch ("stencil" is the full five-field pass; the pressure
# pass of an outer iteration runs the U,V,W-only variant, timed as "stencil_uvw")
KERNEL_OF_STAGE = {"stencil": ("k_stencil", stencil_algo_bytes, stencil_design_bytes),
                   "pface": ("k_pface", pface_algo_bytes, pface_bytes),
                   "mface": ("k_mface", mface_bytes, mface_bytes)}


def fp64_peak_tflops(torch, dev) -> float:
    """FP64 rate of this GPU: cuBLAS DGEMM 4096^3, best of 5 (CUDA events)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    c = a @ b
    best = float("inf")
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def stage_times_alone(ctx, strm, steps: int) -> dict:
    """Per-stage device times of `steps` outer iterations run as their two
    passes called one after the other (calcMomentumEqs, then calcPressureEq:
    the same kernels as semo_outer_iteration, without the pressure setup
    running beside the momentum pass on the second stream).  The kernels'
    rooflines use these: inside the overlapped outer iteration the setup's
    kernels share the multiprocessors with them."""
    ctx.reset_stats()
    ctx.set_profiling(True)
    for _ in range(steps):
        ctx.calc_momentum_eqs()
        ctx.calc_pressure_eq()
    strm.synchronize()
    stages = ctx.stage_times()
    ctx.set_profiling(False)
    return stages


def kernel_rooflines(stages: dict, steps: int, minfo: dict, peak: float, spmv_ms: tuple, levels: list,
                     solve_infos: list) -> dict:
    """HBM fraction of each kernel of an outer iteration that has its own
    stage timer (one launch each), of the two SpMVs timed alone, and of a
    whole CG iteration, from device times and algorithmic bytes."""
    out = {}
    for st, (kname, falgo, _) in KERNEL_OF_STAGE.items():
        ms, calls = stages.get(st, (0.0, 0))
        if calls:
            b = falgo(minfo)
            out[kname] = {"ms": round(ms / calls, 4), "frac": round(b / (ms / calls * 1e-3) / 1e9 / peak, 4)}
    L0 = levels[0]
    b32 = spmv_algo_bytes(L0["rows"], L0["nnz_A"], L0["value_bytes"])
    b64 = spmv_algo_bytes(L0["rows"], L0["nnz_A"], 8)
    out["spmv_level0"] = {"ms": round(spmv_ms[0], 4), "frac": round(b32 / (spmv_ms[0] * 1e-3) / 1e9 / peak, 4)}
    out["spmv_outer_fp64"] = {"ms": round(spmv_ms[1], 4), "frac": round(b64 / (spmv_ms[1] * 1e-3) / 1e9 / peak, 4)}
    it = sum(i["iterations"] for i in solve_infos)
    ms_it = sum(i["solve_ms"] for i in solve_infos) / max(it, 1)
    out["pcg_iteration"] = {"ms": round(ms_it, 4),
                            "frac": round(pcg_iteration_bytes(levels) / (ms_it * 1e-3) / 1e9 / peak, 4)}
    return out


def large_bench(args, S, torch, local) -> dict:
    """The 256^3 jittered VOF case: outer iterations (mixed), then the adjoint
    transpose solve on the same pressure hierarchy; per-kernel HBM fractions
    and the device memory held, against a 180 GB budget."""
    case = bench_case(args.large_n)
    t0 = time.perf_counter()
    ctx = S.Context(precision="mixed", tol=1e-8, device=local, reuse_hierarchy=False)
    ctx.set_case(case)
    t_upload = time.perf_counter() - t0
    minfo = ctx.mesh_info()
    strm = torch.cuda.ExternalStream(ctx.stream, device=torch.device(f"cuda:{local}"))
    for _ in range(2):
        ctx.outer_iteration()
    steps = 3
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(strm)
    infos = [ctx.outer_iteration()[1] for _ in range(steps)]
    e1.record(strm)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    stages = stage_times_alone(ctx, strm, steps)
    spmv_ms = (ctx.time_spmv(0, 20), ctx.time_spmv(1, 20))
    levels = ctx.hierarchy_levels()
    free_b, total_b = torch.cuda.mem_get_info(local)
    used = (total_b - free_b) / 1e9
    # adjoint: J = sum of p'^2 over the z = 1 cells, on the forward hierarchy
    zc = case.mesh.patch_cells("zmax")
    ctx.set_case(case)
    ctx.assemble()
    fwd = ctx.solve()
    g = np.zeros(case.mesh.n_cells)
    np.add.at(g, zc, 2.0 * fwd.x[zc])
    _, _, ainfo = ctx.vjp_source(g)
    ctx.close()
    nc = case.mesh.n_cells
    return {"workload": f"jittered hex {args.large_n}^3 two-phase VOF outer iteration (mixed) + adjoint transpose "
                        f"solve on the same hierarchy",
            "cells": nc, "faces": minfo["faces"], "nnz": minfo["nnz"],
            "value": round(nc / (ms * 1e-3) / 1e6, 3), "unit": UNIT, "ms_per_step": round(ms, 3), "steps": steps,
            "iterations": [i[3]["iterations"] for i in infos], "rel_residual": max(i[3]["rel_residual"] for i in infos),
            "adjoint": {"iterations": ainfo["iterations"], "rel_residual": ainfo["rel_residual"],
                        "adj_over_fwd_krylov": round(ainfo["solve_ms"] / fwd.info["solve_ms"], 3),
                        "ms_adjoint_krylov": round(ainfo["solve_ms"], 3)},
            "device_used_gb": round(used, 2), "budget_gb": 180.0, "upload_s": round(t_upload, 1),
            "amg_levels": len(levels), "level0_layout": levels[0]["layout"],
            "kernels": kernel_rooflines(stages, steps, minfo, hbm_peak()[0], spmv_ms, levels,
                                        [i[3] for i in infos])}


def oracle_outer_iteration(o) -> dict:
    """One outer iteration on the oracle: momentum pass, then pressure pass."""
    m = o.momentum_pass(1e-9)
    o.assemble()
    s = o.solve(False, 1e-8)
    o.update(s["x"])
    return {"mom_iters": m["iters"], "iters": s["iters"]}


def cpu_baseline(case, steps: int = 1):
    """The oracle (restated reference outer iteration) timed on this host's
    cores; returns the baseline object and the oracle after its iteration."""
    from oracle.oracle import Oracle, build
    build()
    o = Oracle(case.mesh)
    o.set_case(case)
    t_total = 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        r = oracle_outer_iteration(o)
        t_total += time.perf_counter() - t0
    n = case.mesh.n_cells
    base = {"value": round(n * steps / t_total / 1e6, 4), "unit": UNIT, "cores": Oracle.threads(),
            "kind": "port", "seconds": round(t_total, 2),
            "sample": f"{steps} outer iteration of the same {n}-cell workload: serial assembly as in SEMO, "
                      f"OpenMP Jacobi-BiCGStab momentum ({r['mom_iters']} iterations) and SA-AMG + CG "
                      f"pressure ({r['iters']} iterations)"}
    return base, o, r


def _relmax(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = float(np.abs(b).max()) if b.size else 0.0
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0)) if a.size else 0.0


def _rel_l2(a, b) -> float:
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


def error_vs_oracle(case, S, local, o_outer, oracle_iters) -> dict:
    """The GPU path against the FP64 CPU oracle on the bench's own workload,
    outside every timed region.

    From the case's fields: the momentum system (CSR pattern in SEMO's layout,
    coefficients, three right-hand sides) and its three solutions; the
    pressure system (RCM CSR pattern, coefficients, right-hand side) and its
    solution (the oracle solves to 1e-12; the GPU to the bench's 1e-8).  Then
    P, U, V, W after one whole outer iteration against the timed oracle run.
    Bars: pattern bit-exact, coefficients and right-hand sides 1e-12 relative
    (max norm), solutions and fields 1e-7 relative L2.
    """
    from oracle.oracle import Oracle
    n = case.mesh.n_cells
    o = Oracle(case.mesh)
    o.set_case(case)
    ctx = S.Context(precision="mixed", tol=1e-8, device=local, reuse_hierarchy=False)
    ctx.set_case(case)
    # momentum: one matrix, three right-hand sides
    ctx.assemble_momentum()
    ms = ctx.momentum_system()
    o.assemble_momentum()
    B = o.get("mom_B").reshape(3, n)
    mom = {"pattern_equal": bool(np.array_equal(ms["ptr"], o.get("mom_csr_ptr"))
                                 and np.array_equal(ms["col"], o.get("mom_csr_col"))),
           "coef_rel": _relmax(ms["val"], o.get("mom_csr_val")),
           "rhs_rel": max(_relmax(ms["b"][j], B[j]) for j in range(3))}
    xg, ig = ctx.solve_momentum()
    xo = o.solve_momentum(1e-12)
    mom["solution_rel_l2"] = max(_rel_l2(xg[j], xo["x"][j]) for j in range(3))
    mom["iterations"] = {"gpu": [i["iterations"] for i in ig], "oracle": list(oracle_iters["mom_iters"])}
    # pressure correction
    ctx.assemble()
    sysm = ctx.system_rcm()
    o.assemble()
    pre = {"pattern_equal": bool(np.array_equal(sysm["ptr"], o.get("rcm_csr_ptr"))
                                 and np.array_equal(sysm["col"], o.get("rcm_csr_col"))),
           "coef_rel": _relmax(sysm["val"], o.get("rcm_csr_val")),
           "rhs_rel": _relmax(sysm["b"], o.get("rcm_B"))}
    res = ctx.solve()
    ref = o.solve(False, 1e-12)
    pre["solution_rel_l2"] = _rel_l2(res.x, ref["x"])
    pre["iterations"] = {"gpu": res.info["iterations"], "oracle": oracle_iters["iters"]}
    pre["rel_residual_gpu"] = res.info["rel_residual"]
    # one whole outer iteration
    ctx.set_case(case)
    ctx.outer_iteration()
    f = ctx.fields()
    outer = {k: _rel_l2(f[k], o_outer.get(k)) for k in ("P", "U", "V", "W")}
    ctx.close()
    ok = (mom["pattern_equal"] and pre["pattern_equal"] and max(mom["coef_rel"], mom["rhs_rel"], pre["coef_rel"],
                                                                 pre["rhs_rel"]) <= 1e-12
          and max(mom["solution_rel_l2"], pre["solution_rel_l2"], *outer.values()) <= 1e-7)
    return {"pass": bool(ok), "momentum": mom, "pressure": pre, "outer_fields_rel_l2": outer,
            "bars": "pattern bit-exact; coefficients, rhs 1e-12 rel (max); solutions, fields 1e-7 rel L2"}


def workload_config(n: int, mesh, world: int) -> dict:
    """The `config` both bench arms print."""
    return {"workload": f"jittered hex {n}^3 two-phase VOF outer iteration: momentum (assembly + 3 BiCGStab "
                        f"solves to 1e-9 + update) then pressure correction (assembly + SA-AMG setup + CG to "
                        f"1e-8 + update)",
            "cells": mesh.n_cells, "faces": mesh.n_faces, "nnz": mesh.n_cells + 2 * mesh.n_internal,
            "parallelism": f"replicas x{world}" if world > 1 else "one device",
            "l2": "inputs larger than L2 (mesh + fields several GB), no flush"}


def bench_case(n: int):
    from semo_mesh_gb300.cases import vof_case, with_history
    return with_history(vof_case(n), seed=5, scale=0.05)


def run_gpu_arm(args, rank, world, local) -> None:
    import torch
    import semo_mesh_gb300 as S
    from semo_mesh_gb300.build import build

    build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    # the clock sampler starts before the case is built (ClockSampler.settle)
    clk = ClockSampler(local).start()
    case = bench_case(args.n)
    mesh = case.mesh
    nc = mesh.n_cells
    inputs = tuple(a.copy() for a in (case.P, case.U, case.V, case.W, case.VF))
    history = case.history()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(ctx, strm, k, fn):
        infos = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(strm)
        for _ in range(k):
            infos.append(fn(ctx)[1])
        e1.record(strm)
        e1.synchronize()
        return e0.elapsed_time(e1) / k, infos

    def outer(ctx):
        return ctx.outer_iteration()

    def pressure(ctx):
        return ctx.calc_pressure_eq()

    # every step rebuilds the AMG hierarchy, as SEMO's solveAMGCL does per call
    ctx = S.Context(precision="mixed", tol=1e-8, device=local, reuse_hierarchy=False)
    ctx.set_case(case)
    minfo = ctx.mesh_info()
    strm = torch.cuda.ExternalStream(ctx.stream, device=torch.device(f"cuda:{local}"))

    # ---- mixed precision, inputs resident in HBM (the headline value) ------
    clk.settle(3.0)
    clk.wait_first()
    for _ in range(args.warmup):
        ctx.outer_iteration()
    l0 = ctx.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    tw0 = time.monotonic()
    ms_mixed, infos = timed(ctx, strm, args.steps, outer)
    torch.cuda.synchronize()
    clk.mark(tw0, time.monotonic())
    time.sleep(0.25)   # one more sample after the window
    clk.stop()
    barrier()
    launches = ctx.kernel_launches() - l0
    # per-stage device times from a second, untimed run of the same steps
    # (stage timers record events on both streams, which costs overlap)
    ctx.reset_stats()
    ctx.set_profiling(True)
    timed(ctx, strm, args.steps, outer)
    stages = ctx.stage_times()
    ctx.set_profiling(False)
    # the kernels alone (no setup beside them), for their rooflines
    stages_alone = stage_times_alone(ctx, strm, args.steps)
    free_b, total_b = torch.cuda.mem_get_info(local)
    used_gb = (total_b - free_b) / 1e9   # the context's mesh, fields, hierarchy and pools, plus torch's own
    if world > 1:
        t = torch.tensor([ms_mixed], device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_mixed = float(t.item())

    # ---- the pressure-correction pass alone (calcPressureEq) ---------------
    ctx.set_case(case)
    for _ in range(args.warmup):
        ctx.calc_pressure_eq()
    ms_pres, infos_p = timed(ctx, strm, args.steps, pressure)
    # where a pressure pass spends its time (a separate, untimed profiled run)
    ctx.reset_stats()
    ctx.set_profiling(True)
    timed(ctx, strm, 3, pressure)
    pstages_mixed = {k: round(v[0] / 3, 4) for k, v in ctx.stage_times().items() if v[1] > 0}
    ctx.set_profiling(False)
    # the apply kernels of the last pass's hierarchy, timed outside the CG graph
    spmv_ms = (ctx.time_spmv(0, 50), ctx.time_spmv(1, 50))
    levels = ctx.hierarchy_levels()

    # ---- one volume-fraction sub-iteration (MSTACS + calcVolfracEq) -------
    ctx.set_case(case)
    for _ in range(args.warmup):
        ctx.calc_volfrac_eq()
    ms_vof, infos_v = timed(ctx, strm, args.steps, lambda cx: cx.calc_volfrac_eq())

    # ---- the pressure pass with multicolour Gauss-Seidel smoothing ----------
    ctxg = S.Context(precision="mixed", tol=1e-8, device=local, reuse_hierarchy=False, smoother="gauss_seidel")
    ctxg.set_case(case)
    strmg = torch.cuda.ExternalStream(ctxg.stream, device=torch.device(f"cuda:{local}"))
    for _ in range(args.warmup):
        ctxg.calc_pressure_eq()
    ms_gs, infos_g = timed(ctxg, strmg, args.steps, pressure)
    ctxg.close()

    # ---- end to end through the C-ABI, host buffers ------------------------
    # inputs and outputs live in pinned host memory, as a caller streaming
    # fields through the library would keep them
    def pinned(a=None):
        t = torch.empty(nc, dtype=torch.float64, pin_memory=True)
        v = t.numpy()
        if a is not None:
            v[:] = a
        return t, v
    pin_in = [pinned(a) for a in inputs]
    h_in = [v for _, v in pin_in]
    pin_hist = [pinned(a) for a in history]
    h_hist = [v for _, v in pin_hist]
    pin_out = {k: pinned() for k in ("P", "U", "V", "W")}
    out = {k: v for k, (_, v) in pin_out.items()}

    def e2e_step():
        ctx.set_fields(*h_in)
        ctx.set_old_velocity(h_hist[:3], h_hist[3:])
        ctx.outer_iteration()
        ctx.fields(out)
    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_t0 = torch.cuda.Event(enable_timing=True)
    e2e_t1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e2e_t0.record(strm)
    for _ in range(args.steps):
        e2e_step()
    e2e_t1.record(strm)
    e2e_t1.synchronize()
    ms_e2e_wall = (time.perf_counter() - t0) * 1e3 / args.steps
    ms_e2e = max(ms_e2e_wall, e2e_t0.elapsed_time(e2e_t1) / args.steps)
    if not np.isfinite(out["P"]).all():
        raise RuntimeError("non-finite pressure after the e2e steps")

    # ---- adjoint: A^T lambda = dJ/dx, J = sum of p'^2 over the z=1 cells -----
    zc = mesh.patch_cells("zmax")
    ctx.set_case(case)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.assemble()
    e0.record(strm)
    fwd = ctx.solve()
    e1.record(strm)
    e1.synchronize()
    ms_fwd = e0.elapsed_time(e1)
    g = np.zeros(nc)
    np.add.at(g, zc, 2.0 * fwd.x[zc])
    e0.record(strm)
    _, _, ainfo = ctx.vjp_source(g)
    e1.record(strm)
    e1.synchronize()
    ms_adj = e0.elapsed_time(e1)
    # the whole field gradient: transpose solve + transposed face-flux kernels
    ctx.vjp_fields(g)
    e0.record(strm)
    _, _, finfo = ctx.vjp_fields(g)
    e1.record(strm)
    e1.synchronize()
    ms_vjpf = e0.elapsed_time(e1)
    ctx.close()

    # ---- hierarchy kept across outer iterations (bit-identical pressure matrix) --
    ctxr = S.Context(precision="mixed", tol=1e-8, device=local, reuse_hierarchy=True)
    ctxr.set_case(case)
    strmr = torch.cuda.ExternalStream(ctxr.stream, device=torch.device(f"cuda:{local}"))
    for _ in range(args.warmup):
        ctxr.outer_iteration()
    ms_reuse, infos_r = timed(ctxr, strmr, args.steps, outer)
    ctxr.close()

    # ---- pressure hierarchy built after the momentum pass, one stream -------
    ctxs = S.Context(precision="mixed", tol=1e-8, device=local, reuse_hierarchy=False, overlap_setup=False)
    ctxs.set_case(case)
    strms = torch.cuda.ExternalStream(ctxs.stream, device=torch.device(f"cuda:{local}"))
    for _ in range(args.warmup):
        ctxs.outer_iteration()
    ms_serial, infos_s = timed(ctxs, strms, args.steps, outer)
    ctxs.close()

    # ---- all-FP64 hierarchy and V-cycle ------------------------------------
    ctx64 = S.Context(precision="fp64", tol=1e-8, device=local, reuse_hierarchy=False)
    ctx64.set_case(case)
    strm64 = torch.cuda.ExternalStream(ctx64.stream, device=torch.device(f"cuda:{local}"))
    for _ in range(args.warmup):
        ctx64.outer_iteration()
    ms_fp64, infos64 = timed(ctx64, strm64, args.steps, outer)
    ctx64.set_case(case)
    for _ in range(args.warmup):
        ctx64.calc_pressure_eq()
    ms_fp64_p, infos64_p = timed(ctx64, strm64, args.steps, pressure)
    ctx64.reset_stats()
    ctx64.set_profiling(True)
    timed(ctx64, strm64, 3, pressure)
    pstages_fp64 = {k: round(v[0] / 3, 4) for k, v in ctx64.stage_times().items() if v[1] > 0}
    ctx64.set_profiling(False)
    ctx64.close()

    # ---- config 4: the 256^3 case, outer iteration and adjoint ---------------
    large = None
    if args.large_n > 0 and world == 1:
        try:
            large = large_bench(args, S, torch, local)
        except S.SemoError as e:   # reported, never allowed to take the headline down
            large = {"error": str(e)}

    # ---- compressible coupled 5x5 system (6 tetrahedra per hex) -------------
    coupled = None
    if args.coupled_n > 0:
        try:
            coupled = coupled_bench(args, S, torch, local)
        except S.SemoError as e:   # reported, never allowed to take the headline down
            coupled = {"error": str(e)}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline for the dominant single-kernel stage ----------------------
    peak, peak_src = hbm_peak()
    fp64_tf = fp64_peak_tflops(torch, torch.device(f"cuda:{local}"))
    single = {k: v for k, v in stages_alone.items() if k in KERNEL_OF_STAGE and v[1] > 0}
    dom = max(single, key=lambda k: single[k][0])   # largest total device time per step
    kname, falgo, fdesign = KERNEL_OF_STAGE[dom]
    per_launch_ms = single[dom][0] / single[dom][1]
    algo = falgo(minfo)
    design = fdesign(minfo)
    achieved = algo / (per_launch_ms * 1e-3) / 1e9
    traffic = None
    fp64_pipe = None
    t = None
    t_all = None
    if os.path.exists(TRAFFIC):
        with open(TRAFFIC) as f:
            tr = json.load(f)
        t_all = tr
        t = tr.get(kname)
        if t and "dram_bytes_per_cell" in t:
            traffic = t["dram_bytes_per_cell"] * nc
        elif t and "dram_bytes_per_launch" in t:
            # hex meshes keep faces/cells fixed, so traffic scales with the faces processed
            traffic = round(t["dram_bytes_per_launch"] * minfo["faces"] / t["faces"])
        if t and "fp64_pipe_pct" in t:
            fp64_pipe = t["fp64_pipe_pct"] / 100.0
    roofline = {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "algorithmic_bytes": algo,
                "design_bytes": design, "ms_per_launch": round(per_launch_ms, 4), "peak_source": peak_src,
                "timed": "CUDA events around the kernel's stage, outer iterations run as their two passes called "
                         "in turn (no pressure setup beside them)"}
    flops = None
    if kname == "k_stencil":
        flops = stencil_fp64_flops(minfo)
    elif t and "dfma_per_launch" in t:
        # the face kernels' FP64 operations (ncu, 64^3) scale with the faces
        flops = (2 * t["dfma_per_launch"] + t["dadd_per_launch"] + t["dmul_per_launch"]) * minfo["faces"] / t["faces"]
    if flops is not None:
        roofline["fp64"] = {"tflops": round(flops / (per_launch_ms * 1e-3) / 1e12, 3),
                            "peak_tflops": round(fp64_tf, 3), "frac": round(flops / (per_launch_ms * 1e-3) / 1e12
                                                                           / fp64_tf, 3),
                            "flops_per_launch": flops, "fp64_pipe_frac_ncu": fp64_pipe,
                            "peak_source": "measured here: cuBLAS DGEMM 4096^3"}
    # the solve: one SpMV of each operator, and a whole CG iteration inside its graph
    L0 = levels[0]
    b32 = spmv_algo_bytes(L0["rows"], L0["nnz_A"], L0["value_bytes"])
    b64 = spmv_algo_bytes(L0["rows"], L0["nnz_A"], 8)
    it_p = sum(i["iterations"] for i in infos_p)
    ms_it = sum(i["solve_ms"] for i in infos_p) / max(it_p, 1)
    pcg_b = pcg_iteration_bytes(levels)
    roofline["spmv_level0"] = {"achieved": round(b32 / (spmv_ms[0] * 1e-3) / 1e9, 1),
                               "frac": round(b32 / (spmv_ms[0] * 1e-3) / 1e9 / peak, 4),
                               "ms_per_launch": round(spmv_ms[0], 4), "algorithmic_bytes": b32,
                               "layout": {2: "SELL-32, 16-bit column offsets", 1: "SELL-32", 0: "CSR"}[L0["layout"]],
                               "value_bytes": L0["value_bytes"]}
    roofline["spmv_outer_fp64"] = {"achieved": round(b64 / (spmv_ms[1] * 1e-3) / 1e9, 1),
                                   "frac": round(b64 / (spmv_ms[1] * 1e-3) / 1e9 / peak, 4),
                                   "ms_per_launch": round(spmv_ms[1], 4), "algorithmic_bytes": b64}
    # DRAM traffic of the two SpMVs (ncu at 128^3), scaled by the nonzeros
    for key, tk in (("spmv_level0", "k_mv_sell16_f32"), ("spmv_outer_fp64", "k_mv_sell16_f64")):
        if t_all and tk in t_all:
            tb = t_all[tk]["dram_bytes_per_launch"] * L0["nnz_A"] / t_all[tk]["nnz"]
            roofline[key]["traffic"] = round(tb)
            roofline[key]["dram_frac"] = round(tb / (roofline[key]["ms_per_launch"] * 1e-3) / 1e9 / peak, 4)
    roofline["pcg_iteration"] = {"achieved": round(pcg_b / (ms_it * 1e-3) / 1e9, 1),
                                 "frac": round(pcg_b / (ms_it * 1e-3) / 1e9 / peak, 4), "ms": round(ms_it, 4),
                                 "algorithmic_bytes": round(pcg_b), "levels": len(levels),
                                 "note": "solve time / iterations of the pressure passes (the graph's iterations "
                                         "plus the initial and final residuals)"}

    cells_all = nc * world
    value = cells_all / (ms_mixed * 1e-3) / 1e6
    clocks = clk.summary()
    mc = lambda ms: round(cells_all / (ms * 1e-3) / 1e6, 3)   # noqa: E731
    # bulky detail first, the summaries last (a reader of the tail sees them)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_mixed, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 assembly + f32 AMG in f64 CG",
        "data": "synthetic (seeded jittered hex mesh, VOF fields, old velocities)",
        "config": workload_config(args.n, mesh, world),
        "gpu_launches": int(launches),
        "clocks": clocks,
        "stages_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in stages.items() if v[1] > 0},
        "pressure_pass_stages_ms": {"mixed": pstages_mixed, "fp64": pstages_fp64},
        "memory": {"device_used_gb": round(used_gb, 2), "device_total_gb": round(total_b / 1e9, 1)},
        "amg_levels": infos[-1][3]["levels"], "operator_complexity": round(infos[-1][3]["operator_complexity"], 3),
        "vof_pass": {"value": mc(ms_vof), "ms_per_step": round(ms_vof, 3),
                     "iterations": [i["iterations"] for i in infos_v][:3],
                     "note": "one volume-fraction sub-iteration (SEMO runs nSpeciesEq of them per time step, "
                             "before its outer iterations)"},
        "serial_setup": {"value": mc(ms_serial), "ms_per_step": round(ms_serial, 3),
                         "overlap_speedup": round(ms_serial / ms_mixed, 3),
                         "note": "the pressure matrix and its hierarchy built after the momentum pass on the one "
                                 "stream; the headline builds them on a second stream during the momentum pass"},
        "hierarchy_reuse": {"value": mc(ms_reuse), "ms_per_step": round(ms_reuse, 3),
                            "iterations": infos_r[-1][3]["iterations"],
                            "setup_ms_last_step": round(infos_r[-1][3]["setup_ms"], 3),
                            "note": "pressure AMG hierarchy kept while the assembled matrix stays bit-identical "
                                    "(outer iterations within a time step); the headline rebuilds it every step"},
    }
    if coupled is not None:
        line["coupled"] = coupled
    if large is not None:
        line["large"] = large
    line.update({
        "roofline": roofline,
        "e2e": {"value": mc(ms_e2e), "unit": UNIT, "ms_per_step": round(ms_e2e, 3),
                "host_buffers": "pinned, caller cell order; semo_set_fields + semo_set_old_velocity + "
                                "semo_outer_iteration + semo_get_fields",
                "h2d_bytes_per_step": 11 * 8 * nc, "d2h_bytes_per_step": 4 * 8 * nc},
        "iterations": [i[3]["iterations"] for i in infos][:3],
        "momentum_iterations": [i[0]["iterations"] for i in infos][:3],
        "rel_residual": max(i[3]["rel_residual"] for i in infos),
        "pressure_pass": {"value": mc(ms_pres), "ms_per_step": round(ms_pres, 3),
                          "iterations": [i["iterations"] for i in infos_p][:3]},
        "smoother_gs": {"ms_per_step": round(ms_gs, 3), "iterations": [i["iterations"] for i in infos_g][:3],
                        "solve_ms": round(sum(i["solve_ms"] for i in infos_g) / len(infos_g), 3),
                        "setup_ms": round(sum(i["setup_ms"] for i in infos_g) / len(infos_g), 3),
                        "chebyshev_solve_ms": round(sum(i["solve_ms"] for i in infos_p) / len(infos_p), 3),
                        "chebyshev_setup_ms": round(sum(i["setup_ms"] for i in infos_p) / len(infos_p), 3),
                        "over_chebyshev": round(ms_gs / ms_pres, 3),
                        "note": "calcPressureEq to 1e-8 with multicolour Gauss-Seidel V(1,1) against the "
                                "headline's Chebyshev V(2,2), both mixed"},
        "fp64": {"value": mc(ms_fp64), "ms_per_step": round(ms_fp64, 3),
                 "iterations": infos64[-1][3]["iterations"], "mixed_speedup": round(ms_fp64 / ms_mixed, 3),
                 "pressure_pass_ms": round(ms_fp64_p, 3),
                 "pressure_pass_mixed_speedup": round(ms_fp64_p / ms_pres, 3)},
        "adjoint": {"ms_adjoint_solve": round(ms_adj, 3), "ms_forward_solve": round(ms_fwd, 3),
                    "adj_over_fwd_krylov": round(ainfo["solve_ms"] / fwd.info["solve_ms"], 3),
                    "adj_over_fwd_solve": round(ms_adj / ms_fwd, 3),
                    "adj_over_fwd_pass": round(ms_adj / ms_pres, 3),
                    "iterations": {"adjoint": ainfo["iterations"], "forward": fwd.info["iterations"]},
                    "ms_vjp_fields": round(ms_vjpf, 3), "vjp_fields_over_pressure_pass": round(ms_vjpf / ms_pres, 3),
                    "note": "krylov: both solves' Krylov time without setup; solve: the forward solve "
                            "includes its AMG setup, the adjoint reuses the hierarchy; vjp_fields: dJ/d(U,V,W,P) "
                            "(transpose solve + transposed face-flux kernels + host copies) against one "
                            "calcPressureEq"},
    })
    if not args.no_cpu_baseline and world == 1:
        base, o_outer, o_iters = cpu_baseline(case, steps=1)
        line["error_vs_oracle"] = error_vs_oracle(case, S, local, o_outer, o_iters)
        line["cpu_baseline"] = base
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def coupled_bench(args, S, torch, local) -> dict:
    """calcCompCoupledEq on the tetrahedral ideal-gas case, FP64 and mixed.

    A step is one coupled pass (EOS, gradients, 5x5 block assembly, solve to
    a 1e-8 FP64 relative residual, update) from the case's fields: the
    fields are put back between steps (outside the timed region; each pass
    is timed with CUDA events on the context's stream), so every step solves
    the same system."""
    from semo_mesh_gb300.cases import coupled_case
    case = coupled_case(args.coupled_n)
    m = case.mesh
    steps = min(args.steps, 5)
    out = {"workload": f"6 tets per hex of a jittered {args.coupled_n}^3 box, ideal gas, config-2 fields, dt 1e-5; "
                       "one calcCompCoupledEq to 1e-8",
           "cells": m.n_cells, "faces": m.n_faces, "block_slots": m.n_cells + 2 * m.n_internal, "steps": steps}
    for prec in ("fp64", "mixed"):
        ctx = S.Context(precision=prec, tol=1e-8, max_iter=3000, device=local)
        ctx.set_coupled_case(case)
        strm = torch.cuda.ExternalStream(ctx.stream, device=torch.device(f"cuda:{local}"))
        fields = (case.P, case.U, case.V, case.W, case.T, *case.history())
        for _ in range(args.warmup):
            ctx.set_coupled_fields(*fields)
            ctx.calc_comp_coupled_eq()
        ctx.set_profiling(True)
        ctx.reset_stats()
        infos, total = [], 0.0
        for _ in range(steps):
            ctx.set_coupled_fields(*fields)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(strm)
            infos.append(ctx.calc_comp_coupled_eq()[1])
            e1.record(strm)
            e1.synchronize()
            total += e0.elapsed_time(e1)
        ms = total / steps
        st = ctx.stage_times()
        free_b, total_b = torch.cuda.mem_get_info()
        out[prec] = {"value": round(m.n_cells / (ms * 1e-3) / 1e6, 3), "unit": UNIT, "ms_per_step": round(ms, 3),
                     "iterations": [i["iterations"] for i in infos], "outer_steps": infos[-1]["levels"],
                     "rel_residual": infos[-1]["rel_residual"],
                     "stages_ms_per_step": {k: round(v[0] / steps, 3) for k, v in st.items() if v[1] > 0},
                     "device_used_gb": round((total_b - free_b) / 1e9, 2)}
        ctx.close()
    out["mixed_speedup"] = round(out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"], 3)
    # what bounds one FP64 block product: 25 FMAs per 200-byte block
    slots = out["block_slots"]
    out["block_product_bound"] = {
        "hbm_ms": round(slots * (200 + 4 + 40) / (hbm_peak()[0] * 1e9) * 1e3, 3),
        "fp64_ms": round(slots * 50 / 1.26e12 * 1e3, 3),
        "note": "FP64 block product: 25 FMAs per 200-byte block; at this part's FP64 rate (1.26 TFLOP/s, measured "
                "with independent FMA chains) the arithmetic takes longer than the bytes"}
    return out


def run_reference_arm(args, rank, world) -> None:
    """The reference's CPU implementation of the path (oracle port), same workload."""
    if rank != 0:
        return
    from oracle.oracle import Oracle, build
    build()
    case = bench_case(args.n)
    o = Oracle(case.mesh)
    o.set_case(case)
    times, iters = [], []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = oracle_outer_iteration(o)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            iters.append(r["iters"])
    nc = case.mesh.n_cells
    ms = 1e3 * sum(times) / len(times)
    value = nc / (ms * 1e-3) / 1e6
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded jittered hex mesh, VOF fields, old velocities)",
            "impl": "reference",
            "config": workload_config(args.n, case.mesh, world),
            "iterations": iters[:3],
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": Oracle.threads(), "kind": "port",
                             "sample": f"each step one full outer iteration over all {nc} cells on the host cores"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=128, help="hex cells per edge")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--coupled-n", type=int, default=96,
                    help="hexes per edge of the tetrahedral coupled case (0 skips it)")
    ap.add_argument("--large-n", type=int, default=256,
                    help="hex cells per edge of the large VOF case (0 skips it)")
    ap.add_argument("--coupled-only", action="store_true",
                    help="run only the coupled case and print its object (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
    elif args.coupled_only:
        import torch
        import semo_mesh_gb300 as S
        from semo_mesh_gb300.build import build
        build()
        torch.cuda.set_device(local)
        print(json.dumps({"coupled": coupled_bench(args, S, torch, local)}), flush=True)
    else:
        run_gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
