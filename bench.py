"""Benchmark of the Wilson-twisted-mass hot path on one GB300 (or N replicas).

Workload (one "step" = one application of the FP64 Wilson-Dirac operator
D on a 24^3 x 48 lattice, kappa = 0.150, antiperiodic in t, synthetic SU(3)
links with mean plaquette 0.60 and a seeded Gaussian spinor): the lattice of
the plain FP64 single-RHS configuration, timed over K applications.

  value  -- device-resident: algorithmic bytes per apply (spinor in + 4
            links (18 reals) + spinor out = 960 B/site) / kernel time, GB/s,
            for the faster FP64-accurate kernel (float-float or native).
  e2e    -- the same apply through the qcd_lib C entry point
            qcd_applyWilsonTMOp on host (page-locked) buffers: each step
            copies the input spinor host->device and the result back; the
            gauge field is uploaded once beforehand (qcdgpu_gauge_upload).
  solve  -- point-source columns at 24^3 x 48 to a true residual of 1e-10:
            plain FP64 GPU CGNR (the drop-in) vs mixed precision and even/odd.
  precision_32x64 -- the same comparison at 32^3 x 64, kappa = 0.155, plus
            batched multi-RHS solves (full and even/odd).
  mrhs_operator -- multi-RHS operator at 48^3 x 96 over RHS per block.
  serving -- a seeded Poisson stream of requests (four resident gauge
            fields, 8^3 x 16 ... 32^3 x 64, 1-48 RHS each): RHS-solves/s and
            p50 / p99 latency.

Multi-GPU: the operator keeps the whole lattice on one GPU; N processes run
N independent replicas (no collective) and value sums their throughput.

--impl reference times the reference's CPU path (the oracle build of the
reference where it exists, else the C restatement) on all host cores.
--only X runs one part alone (the profiling targets of profiles/).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L_BENCH = (48, 24, 24, 24)  # t, x, y, z
KAPPA = 0.150
L_PREC, KAPPA_PREC = (64, 32, 32, 32), 0.155  # precision / batching comparison
L_MRHS = (96, 48, 48, 48)  # multi-RHS operator sweep
THETA = (3.141592653589793, 0.0, 0.0, 0.0)
EPS_PLAQ_060 = 0.43374
FLOPS_PER_SITE = 1320
METRIC = "Dslash GB/s (% HBM peak); RHS-solves/s, p99 latency @1e-10 vs plain FP64 GPU"


def bytes_per_site(prec: int, recon: int) -> int:
    """compulsory HBM bytes per site of one apply: spinor in, 4 links, spinor out"""
    if prec == 0:
        return 192 + 4 * recon * 8 + 192
    if prec == 1:
        return 96 + 4 * recon * 4 + 96
    return 52 + 4 * 12 * 2 + 52


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


def profile_value(name: str, key: str = "dram_bytes_per_launch"):
    """a figure of the committed ncu summary (`key: value` line), if present"""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":")[1])
    return None


def profile_traffic(name: str):
    """DRAM bytes per launch from the committed ncu summary, if present"""
    return profile_value(name)


def compute_ceiling(q, V, ms_native, ms_df64, sm_mhz):
    """the FP64 operator against its arithmetic ceilings: the native kernel
    against the FP64 FMA pipe (1320 flops per site at the FMA rate measured
    here), the float-float kernel against instruction issue (its warp
    instructions per apply from the committed ncu capture, four warp
    instructions per clock per SM at the sampled SM clock)"""
    import ctypes as C

    out = {}
    r64, r32 = C.c_double(), C.c_double()
    if q.lib().qcdgpu_measure_fma_rate(0, C.byref(r64)) == 0 and ms_native:
        floor = V * FLOPS_PER_SITE / (r64.value * 1e12) * 1e3
        out["native_fp64"] = {"bound": "fp64 fma pipe", "fp64_tflops_measured": r64.value,
                              "flops_per_site": FLOPS_PER_SITE, "floor_ms": floor, "kernel_ms": ms_native,
                              "frac": floor / ms_native}
    if q.lib().qcdgpu_measure_fma_rate(1, C.byref(r32)) == 0:
        out["fp32_tflops_measured"] = r32.value
    instr = profile_value("dslash_df64_24x24x24x48.md", "warp_instructions_per_launch")
    if instr and ms_df64:
        import torch

        sms = torch.cuda.get_device_properties(0).multi_processor_count
        mhz = sm_mhz or 2070.0
        floor = instr / (4.0 * sms * mhz * 1e6) * 1e3
        out["float_float"] = {"bound": "instruction issue", "warp_instructions": instr, "sm_mhz": mhz,
                              "floor_ms": floor, "kernel_ms": ms_df64, "frac": floor / ms_df64,
                              "hbm_floor_ms": None}
    return out


class ClockSampler:
    """samples nvidia-smi SM clocks and throttle reasons in the background"""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline
def _cpu_worker(args):
    """one process: time the oracle's FP64 operator on the bench lattice"""
    budget_s, L = args
    import numpy as np

    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle

    orc = Oracle()
    u = orc.gauge_synthetic(L, 0, EPS_PLAQ_060)
    v = orc.gaussian_spinor(L, 1)
    out = np.empty_like(v)
    orc.dslash_fast(v, u, L, THETA, kappa=KAPPA, out=out)  # builds the neighbour tables (untimed)
    n = 0
    t0 = time.perf_counter()
    while True:
        orc.dslash_fast(v, u, L, THETA, kappa=KAPPA, out=out)
        n += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    return n, time.perf_counter() - t0


def cpu_baseline(budget_s: float, procs: int, L=L_BENCH) -> dict:
    import multiprocessing as mp

    from oracle.oracle import ORACLE_SO, build

    if not os.path.exists(ORACLE_SO):
        build(with_ref=False)
    V = L[0] * L[1] * L[2] * L[3]
    ctx = mp.get_context("spawn")
    if procs == 1:
        res = [_cpu_worker((budget_s, L))]
    else:
        with ctx.Pool(procs) as pool:
            res = pool.map(_cpu_worker, [(budget_s, L)] * procs)
    rate = sum(n / t for n, t in res)  # applies per second, all processes
    gbs = rate * V * bytes_per_site(0, 18) / 1e9
    applies = sum(n for n, _ in res)
    return {"value": gbs, "unit": "GB/s", "cores": procs, "kind": "port",
            "sample": f"{applies} FP64 D applies of {L[3]}^3x{L[0]} ({budget_s:.0f} s per process, "
                      f"{procs} process(es)); the timed code restates qcd_applyWilsonTMOp's half-spinor "
                      f"algorithm (project, multiply the half spinor, rebuild; plus/minus site tables) at -O3, "
                      f"within 15% of the reference's own compiled function on one core (tested)",
            "applies_per_s": rate}


def config1_solves(q, budget_s: float) -> dict:
    """The reference's CPU-runnable case: point-source columns on 8^3x16,
    kappa 0.150, solved to a true residual of 1e-10. CPU: the C restatement's
    FP64 CGNR on one host core, as many columns as fit the time budget (at
    least one). GPU: all 12 columns, even/odd CGNR with FP16 inner iterations
    and plain FP64 CGNR, and the configuration's BiCGstab: BiCGstab(8) on the
    even/odd system with FP64 and with FP32 inner iterations (plain BiCGstab
    stagnates near 5e-3 on this ensemble at kappa 0.150). Identical inputs on
    both sides."""
    import numpy as np

    from oracle.oracle import Oracle

    orc = Oracle()
    L = (16, 8, 8, 8)
    V = L[0] * L[1] * L[2] * L[3]
    u = orc.gauge_synthetic(L, 0, EPS_PLAQ_060)

    def point(col):
        b = np.zeros((V, 4, 3, 2))
        b[0, col // 3, col % 3, 0] = 1.0
        return b

    # the restatement's CGNR stops on the normal equations' residual: find
    # (untimed, on column 0) the tolerance that gives a true residual <= 1e-10
    tol_ne = 1e-10
    while tol_ne > 1e-14:
        x, _, _ = orc.cgnr(point(0), u, L, THETA, KAPPA, tol=tol_ne)
        if orc.true_residual(x, point(0), u, L, THETA, KAPPA) <= 1e-10:
            break
        tol_ne *= 0.5
    cols, iters, cpu_res = 0, [], 0.0
    t0 = time.perf_counter()
    while cols < 12:
        x, it, _ = orc.cgnr(point(cols), u, L, THETA, KAPPA, tol=tol_ne)
        iters.append(int(it))
        cols += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    cpu_s = time.perf_counter() - t0
    cpu_res = orc.true_residual(x, point(cols - 1), u, L, THETA, KAPPA)
    g = q.Gauge(L, THETA).load(u)
    out = {"lattice_txyz": list(L), "kappa": KAPPA, "tol": 1e-10,
           "cpu_fp64_cgnr": {"rhs_solves_per_s": cols / cpu_s, "columns": cols, "iters": iters, "cores": 1,
                             "kind": "port", "true_residual_last": cpu_res, "normal_eq_tol": tol_ne}}
    for name, solver, prec in (("gpu_eo_cgnr_f16", q.SOLVER_CGNR_EO, q.F16), ("gpu_fp64_cgnr", q.SOLVER_CGNR, q.F64),
                               ("gpu_eo_bicgstab8_f64", q.SOLVER_BICGSTABL_EO, q.F64),
                               ("gpu_eo_bicgstab8_f32", q.SOLVER_BICGSTABL_EO, q.F32)):
        xs = [q.Field(L) for _ in range(12)]
        bs = [q.Field(L).point((0, 0, 0, 0), c // 3, c % 3) for c in range(12)]
        q.solve(xs[0], bs[0], g, KAPPA, 0.0, solver=solver, inner_prec=prec, tol=1e-10, restart=8,
                maxiter=40000)  # warm-up
        q.sync()
        t0 = time.perf_counter()
        ps = [q.solve(xs[c], bs[c], g, KAPPA, 0.0, solver=solver, inner_prec=prec, tol=1e-10, restart=8,
                      maxiter=40000) for c in range(12)]
        q.sync()
        dt = time.perf_counter() - t0
        res = max(orc.true_residual(xs[c].store(), point(c), u, L, THETA, KAPPA) for c in range(12))
        out[name] = {"rhs_solves_per_s": 12 / dt, "columns": 12, "iters": [p.iters for p in ps],
                     "max_true_residual": res, "status": sorted({p.status for p in ps})}
        for f in xs + bs:
            f.close()
    # the reference's own solver: GCR(32) on Q = i g5 D (invert.c:20-113, first
    # basis term restored), one cycle of 32 steps on the GPU (batched
    # Gram-Schmidt) and on one host core (the C restatement); the true residual
    # after ten cycles of the drop-in's restarts
    geo = q.Geometry(L, THETA)
    src, sol, gfd = q.Vector(geo), q.Vector(geo), q.GaugeField(geo)
    gfd.a[:] = u
    src.a[:] = point(0)
    lib = q.lib()
    lib.gcr(sol.ref, src.ref, gfd.ref, KAPPA, 0.0, 32, geo.s)  # warm-up
    t0 = time.perf_counter()
    for _ in range(3):
        lib.gcr(sol.ref, src.ref, gfd.ref, KAPPA, 0.0, 32, geo.s)
    gpu_cycle = (time.perf_counter() - t0) / 3
    t0 = time.perf_counter()
    orc.gcr(point(0), u, L, THETA, KAPPA, 0.0, 32, fixed=True)
    cpu_cycle = time.perf_counter() - t0
    xg = q.Field(L)
    bg = q.Field(L).load(point(0))
    p10 = q.solve(xg, bg, g, KAPPA, 0.0, solver=q.SOLVER_GCR, op=q.OP_Q, tol=1e-10, restart=32, maxiter=320)
    out["gcr32"] = {"gpu_ms_per_cycle": 1e3 * gpu_cycle, "cpu_ms_per_cycle_1core": 1e3 * cpu_cycle,
                    "speedup": cpu_cycle / gpu_cycle, "true_residual_after_10_cycles": p10.true_residual,
                    "note": "32 GCR steps on Q per cycle, Gram-Schmidt as one multi-dot and one batched axpy per step; "
                            "the CPU cycle is the C restatement (the checker build, general gamma matrices)"}
    for o in (src, sol, gfd, xg, bg):
        o.close()
    geo.close()
    g.close()
    out["speedup_gpu_eo_f16_vs_cpu_1core"] = out["gpu_eo_cgnr_f16"]["rhs_solves_per_s"] / out["cpu_fp64_cgnr"]["rhs_solves_per_s"]
    return out


# ------------------------------------------------------------ replicas
def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """the largest x over all ranks (replicas time their own work; the job's
    time is the slowest replica's)"""
    if world <= 1:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(bytes_per_step_per_rank: float, ms_max: float, world: int) -> float:
    """whole-job GB/s: every replica moves the same bytes per step, the job
    takes the slowest replica's time"""
    return bytes_per_step_per_rank * world / (ms_max * 1e-3) / 1e9


# ------------------------------------------------------------- GPU parts
def time_dslash(q, torch, fout, fin, g, steps, warmup, arith, stream):
    lib = q.lib()
    for _ in range(warmup):
        q.dslash(fout, fin, g, KAPPA, 0.0, q.OP_D, arith)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = lib.qcdgpu_kernel_launches()
    start.record(stream)
    for _ in range(steps):
        q.dslash(fout, fin, g, KAPPA, 0.0, q.OP_D, arith)
    stop.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / steps, lib.qcdgpu_kernel_launches() - n0


def time_e2e(q, torch, steps, warmup, u_host, v_host):
    """qcd_applyWilsonTMOp on host buffers; returns ms per step and bytes"""
    import numpy as np

    lib = q.lib()
    geo = q.Geometry(L_BENCH, THETA)
    u, v, Dv = q.GaugeField(geo), q.Vector(geo), q.Vector(geo)
    u.a[:] = u_host
    v.a[:] = v_host
    assert lib.qcdgpu_gauge_upload(u.ref) == 0
    m = 1.0 / (2.0 * KAPPA) - 4.0
    for _ in range(warmup):
        assert lib.qcd_applyWilsonTMOp(Dv.ref, v.ref, u.ref, m, 0.0) == 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        assert lib.qcd_applyWilsonTMOp(Dv.ref, v.ref, u.ref, m, 0.0) == 0
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    out = np.array(Dv.a[:4])
    nbytes = geo.V * 192
    for o in (u, v, Dv):
        o.close()
    geo.close()
    return ms, nbytes, nbytes, out


def solve_bench(q, orc_check, g, L, n_rhs):
    """point-source columns solved to 1e-10: plain FP64 vs mixed precision"""
    out = {}
    b, x = q.Field(L), q.Field(L)
    for name, solver, prec in (("fp64_cgnr", q.SOLVER_CGNR, q.F64), ("mixed_cgnr_f16", q.SOLVER_CGNR, q.F16),
                               ("mixed_cgnr_f32", q.SOLVER_CGNR, q.F32), ("eo_cgnr_f32", q.SOLVER_CGNR_EO, q.F32),
                               ("eo_cgnr_f16", q.SOLVER_CGNR_EO, q.F16)):
        lat, iters, res, status = [], [], [], []
        for col in range(n_rhs):
            b.point((0, 0, 0, 0), col // 3, col % 3)
            q.sync()
            t0 = time.perf_counter()
            p = q.solve(x, b, g, KAPPA, 0.0, solver=solver, inner_prec=prec, tol=1e-10)
            q.sync()
            lat.append(time.perf_counter() - t0)
            iters.append(p.iters)
            res.append(p.true_residual)
            status.append(p.status)
        lat.sort()
        ok = all(s == 0 for s in status)
        out[name] = {"rhs_solves_per_s": n_rhs / sum(lat) if ok else None, "p50_ms": 1e3 * lat[len(lat) // 2],
                     "p99_ms": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))], "iters": iters,
                     "max_true_residual": max(res), "status": status}
    if out["fp64_cgnr"]["rhs_solves_per_s"]:
        for k in ("mixed_cgnr_f16", "mixed_cgnr_f32", "eo_cgnr_f32", "eo_cgnr_f16"):
            if out[k]["rhs_solves_per_s"]:
                out["speedup_" + k + "_vs_fp64"] = out[k]["rhs_solves_per_s"] / out["fp64_cgnr"]["rhs_solves_per_s"]
    # the configuration's own source: a point at the origin, Gaussian-smeared
    # (alpha 4.0, 50 steps) on APE-smeared links (alpha 0.5, 20 steps), built
    # on the GPU; the solve runs on the unsmeared links
    sm = {}
    for spin_col in range(2):
        q.smeared_source(b, g, (0, 0, 0, 0), spin_col, spin_col, 0.5, 20, 4.0, 50)
        for name, solver, prec in (("fp64_cgnr", q.SOLVER_CGNR, q.F64), ("eo_cgnr_f16", q.SOLVER_CGNR_EO, q.F16)):
            q.sync()
            t0 = time.perf_counter()
            p = q.solve(x, b, g, KAPPA, 0.0, solver=solver, inner_prec=prec, tol=1e-10)
            q.sync()
            d = sm.setdefault(name, {"s": [], "iters": [], "true_residual": [], "status": []})
            d["s"].append(time.perf_counter() - t0)
            d["iters"].append(p.iters)
            d["true_residual"].append(p.true_residual)
            d["status"].append(p.status)
    for d in sm.values():
        ok = all(st == 0 for st in d["status"])
        d["rhs_solves_per_s"] = len(d["s"]) / sum(d["s"]) if ok else None
    if sm["fp64_cgnr"]["rhs_solves_per_s"] and sm["eo_cgnr_f16"]["rhs_solves_per_s"]:
        sm["speedup_eo_cgnr_f16_vs_fp64"] = sm["eo_cgnr_f16"]["rhs_solves_per_s"] / sm["fp64_cgnr"]["rhs_solves_per_s"]
    sm["source"] = "point at the origin, Gaussian alpha 4.0 x 50 on APE alpha 0.5 x 20 links (two spin-colour columns)"
    out["smeared_source"] = sm
    b.close()
    x.close()
    return out


def mrhs_bench(q, torch, stream, L, nrhs_list, steps):
    """multi-RHS operator (FP16 spinors, one link read per site for all RHS):
    time per apply and algorithmic GB/s for each RHS-per-block count"""
    V = L[0] * L[1] * L[2] * L[3]
    g = q.Gauge(L, THETA).synthetic(3, EPS_PLAQ_060)
    f = q.Field(L)
    rows = []
    for N in nrhs_list:
        mi, mo = q.MField(L, N), q.MField(L, N)
        for r in range(N):
            mi.set(r, f.gaussian(500 + r))
        for _ in range(3):  # the first call tunes the kernel variant for (V, N)
            q.dslash_mrhs(mo, mi, g, KAPPA, 0.0, q.OP_D, N)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            q.dslash_mrhs(mo, mi, g, KAPPA, 0.0, q.OP_D, N)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        byts = V * (N * 104 + 288)  # N x (FP16 spinor + norm, in and out) + 4 FP32 links once per site
        rows.append({"rhs_per_block": N, "ms_per_apply": ms, "us_per_rhs_apply": 1e3 * ms / N,
                     "gbs": byts / (ms * 1e-3) / 1e9, "tuned": q.mrhs_tuned(L, N),
                     "gflops": V * N * FLOPS_PER_SITE / (ms * 1e-3) / 1e9})
        mi.close()
        mo.close()
    g.close()
    f.close()
    return {"lattice_txyz": list(L), "bytes_per_site": "104 * N + 288", "sweep": rows}


def precision_bench(q, L, kappa, n_batch, cap):
    """point-source columns at L, kappa, to a true residual of 1e-10: the plain
    FP64 GPU solve (one RHS at a time) against single-RHS mixed precision and
    the batched multi-RHS solver; RHS-solves/s over the same columns"""
    out = {"lattice_txyz": list(L), "kappa": kappa, "tol": 1e-10}
    g = q.Gauge(L, THETA).synthetic(2, EPS_PLAQ_060)
    b, x = q.Field(L), q.Field(L)
    for name, solver, prec in (("fp64_cgnr", q.SOLVER_CGNR, q.F64), ("mixed_cgnr_f32", q.SOLVER_CGNR, q.F32),
                               ("mixed_cgnr_f16", q.SOLVER_CGNR, q.F16), ("eo_cgnr_f32", q.SOLVER_CGNR_EO, q.F32),
                               ("eo_cgnr_f16", q.SOLVER_CGNR_EO, q.F16)):
        b.point((0, 0, 0, 0), 0, 0)
        q.sync()
        t0 = time.perf_counter()
        p = q.solve(x, b, g, kappa, 0.0, solver=solver, inner_prec=prec, tol=1e-10, maxiter=40000)
        q.sync()
        dt = time.perf_counter() - t0
        out[name] = {"rhs_solves_per_s": 1.0 / dt if p.status == 0 else None, "s_per_solve": dt, "iters": p.iters,
                     "reliable_updates": p.reliable_updates, "true_residual": p.true_residual, "status": p.status}
    srcs = [q.Field(L).point((0, 0, 0, 0), c % 12 // 3, c % 3) if c < 12 else
            q.Field(L).point((L[0] // 2, (c // 12) % L[1], 0, 0), c % 12 // 3, c % 3) for c in range(n_batch)]
    xs = [q.Field(L) for _ in range(n_batch)]
    for name, eo in (("batched_mrhs", False), ("batched_mrhs_eo", True)):
        batch = q.Batch(g, cap, eo=eo)
        q.sync()
        t0 = time.perf_counter()
        queue = list(range(n_batch))
        done = []
        lat = {}
        while queue or batch.active:
            while queue and batch.free_slots > 0:
                c = queue.pop(0)
                batch.add(xs[c], srcs[c], kappa, 0.0, q.OP_D, tol=1e-10, maxiter=40000, tag=c)
            batch.step(16)
            for d in batch.poll():
                done.append(d)
                lat[d[0]] = time.perf_counter() - t0
        q.sync()
        dt = time.perf_counter() - t0
        ok = len(done) == n_batch and all(d[1] == 0 for d in done)
        ls = sorted(lat.values())
        out[name] = {"rhs": n_batch, "slots": cap, "rhs_solves_per_s": n_batch / dt if ok else None,
                     "wall_s": dt, "iters_max": max(d[2] for d in done), "iters_min": min(d[2] for d in done),
                     "max_true_residual": max(d[3] for d in done), "status": sorted({d[1] for d in done}),
                     "p50_s": ls[len(ls) // 2], "p99_s": ls[min(len(ls) - 1, int(0.99 * len(ls)))],
                     "tuned": None if eo else q.mrhs_tuned(L, cap)}
        batch.close()
    base = out["fp64_cgnr"]["rhs_solves_per_s"]
    if base:
        for k in ("mixed_cgnr_f32", "mixed_cgnr_f16", "eo_cgnr_f32", "eo_cgnr_f16"):
            if out[k]["rhs_solves_per_s"]:
                out["speedup_" + k + "_vs_fp64"] = out[k]["rhs_solves_per_s"] / base
        for k in ("batched_mrhs", "batched_mrhs_eo"):
            if out[k]["rhs_solves_per_s"]:
                out["speedup_" + k + "_vs_fp64"] = out[k]["rhs_solves_per_s"] / base
    for f in srcs + xs + [g, b, x]:
        f.close()
    return out


def batching_bench(q, L, kappa, nrhs, caps=(4, 8, 16, 32), sweep_rhs=32):
    """The batching configuration at L (48^3 x 96), kappa: nrhs right-hand
    sides = 8 source positions x 12 spin-colour columns, solved to 1e-10 by
    even/odd batches with continuous admission. First the RHS-per-block sweep
    inside the solve (the first sweep_rhs columns at each batch capacity in
    caps; at 32 per block the batch holds ~100 GB and the 32 pairs of FP64 x
    and b in flight ~131 GB), then all nrhs columns at the fastest capacity.
    Beside them one even/odd FP16 solve and one plain FP64 solve of the first
    column."""
    g = q.Gauge(L, THETA).synthetic(4, EPS_PLAQ_060)
    out = {"lattice_txyz": list(L), "kappa": kappa, "rhs": nrhs, "tol": 1e-10,
           "sources": "points at t in {0, L_t/2} x (x, y, z) in {0, (L/2,0,0), (0,L/2,0), (0,0,L/2)}, 12 columns each"}
    b, x = q.Field(L), q.Field(L)
    for name, solver, prec in (("fp64_cgnr", q.SOLVER_CGNR, q.F64), ("eo_cgnr_f16", q.SOLVER_CGNR_EO, q.F16)):
        b.point((0, 0, 0, 0), 0, 0)
        q.sync()
        t0 = time.perf_counter()
        p = q.solve(x, b, g, kappa, 0.0, solver=solver, inner_prec=prec, tol=1e-10, maxiter=40000)
        q.sync()
        dt = time.perf_counter() - t0
        out[name] = {"rhs_solves_per_s": 1.0 / dt if p.status == 0 else None, "s_per_solve": dt, "iters": p.iters,
                     "true_residual": p.true_residual, "status": p.status}
    b.close()
    x.close()
    h = L[1] // 2
    spatial = ((0, 0, 0), (h, 0, 0), (0, h, 0), (0, 0, h))
    positions = [(t, *xyz) for t in (0, L[0] // 2) for xyz in spatial]

    def run(cap, n):
        """columns 0..n-1 through an even/oddbatch of cap slots; x and b
        fields are taken from a pool of cap pairs and returned on retirement"""
        pool = [(q.Field(L), q.Field(L)) for _ in range(cap)]
        free = list(range(cap))
        batch = q.Batch(g, cap, eo=True)
        busy, done = {}, []
        q.sync()
        t0 = time.perf_counter()
        c = 0
        while c < n or batch.active:
            while c < n and free:
                k = free.pop()
                xf, bf = pool[k]
                pos = positions[(c // 12) % len(positions)]
                bf.point(pos, c % 12 // 3, c % 3)
                batch.add(xf, bf, kappa, 0.0, q.OP_D, tol=1e-10, maxiter=40000, tag=c)
                busy[c] = k
                c += 1
            batch.step(16)
            for d in batch.poll():
                done.append(d)
                free.append(busy.pop(d[0]))
        q.sync()
        dt = time.perf_counter() - t0
        nbytes = batch.nbytes()
        batch.close()
        for xf, bf in pool:
            xf.close()
            bf.close()
        ok = len(done) == n and all(d[1] == 0 for d in done)
        return {"slots": cap, "rhs": n, "rhs_solves_per_s": n / dt if ok else None, "wall_s": dt,
                "iters_max": max(d[2] for d in done), "max_true_residual": max(d[3] for d in done),
                "status": sorted({d[1] for d in done}), "batch_bytes": nbytes}

    sweep = []
    for cap in caps:
        q.release_work()
        sweep.append(run(cap, sweep_rhs))
    out["rhs_per_block_sweep"] = sweep
    ok = [r for r in sweep if r["rhs_solves_per_s"]]
    best = max(ok, key=lambda r: r["rhs_solves_per_s"])["slots"] if ok else caps[-1]
    q.release_work()
    out["batched_mrhs_eo"] = run(best, nrhs)
    base = out["fp64_cgnr"]["rhs_solves_per_s"]
    if base and out["batched_mrhs_eo"]["rhs_solves_per_s"]:
        out["speedup_batched_mrhs_eo_vs_fp64"] = out["batched_mrhs_eo"]["rhs_solves_per_s"] / base
    g.close()
    return out


def serving_bench(q, seconds, rate, slots, budget_gb, weights=None):
    """Poisson stream over four resident gauge fields (one per volume); with
    weights, requests draw the volumes with those weights"""
    from qcd_gb300 import serving

    gauges = serving.build_gauges()
    srv = q.Server(int(budget_gb * 2**30), slots)
    ids = [srv.add_gauge(g) for g in gauges]
    arr = serving.make_stream(rate, seconds, len(ids), seed=7, weights=weights)
    res = serving.run_stream(srv, ids, arr, max_wall_s=seconds * 6 + 60)
    res.update({"rate_hz": rate, "arrival_s": seconds, "slots": slots, "budget_gb": budget_gb, "volume_weights": weights,
                "volumes_txyz": [list(L) for L in serving.SERVE_VOLUMES], "kappa": [0.14, 0.155],
                "rhs_per_request": [1, 48], "tols": [1e-8, 1e-10]})
    srv.close()
    for g in gauges:
        g.close()
    return res


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import qcd_gb300 as q

    torch.cuda.set_device(local_rank)
    stream = torch.cuda.current_stream()
    q.set_stream(stream.cuda_stream)
    V = L_BENCH[0] * L_BENCH[1] * L_BENCH[2] * L_BENCH[3]
    g = q.Gauge(L_BENCH, THETA).synthetic(1000 + rank, EPS_PLAQ_060)
    plaq = g.plaquette()
    fin, fout = q.Field(L_BENCH).gaussian(2000 + rank), q.Field(L_BENCH)
    recon = g.recon
    bps = bytes_per_site(0, 18)  # FP64 kernels read complete links (arithmetic-bound, no rebuild)
    sampler = ClockSampler(local_rank)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms_native, launches = time_dslash(q, torch, fout, fin, g, args.steps, args.warmup, q.ARITH_F64, stream)
    ms_df64 = None
    try:
        ms_df64, launches_df = time_dslash(q, torch, fout, fin, g, args.steps, args.warmup, q.ARITH_DF64, stream)
    except q.QcdGpuError:
        ms_df64 = None
    clocks = sampler.stop()
    # fastest FP64-accurate kernel is the product path
    best_ms, arith = (ms_native, "f64") if ms_df64 is None or ms_native <= ms_df64 else (ms_df64, "df64")
    if arith == "df64":
        launches = launches_df
    ms_max = max_over_ranks(best_ms, world)
    # e2e through the C entry point with host buffers
    u_host = g.store()
    v_host = fin.store()
    q.lib().qcdgpu_set_f64_arith(q.ARITH_DF64 if arith == "df64" else q.ARITH_F64)
    e2e_steps = max(3, min(args.steps, 50))
    ms_e2e, h2d, d2h, _ = time_e2e(q, torch, e2e_steps, max(1, args.warmup // 4), u_host, v_host)
    solve = None
    if not args.no_solve and rank == 0:
        solve = solve_bench(q, None, g, L_BENCH, args.solve_rhs)
    for f in (g, fin, fout):
        f.close()
    mrhs = precision = serving = batching = None
    if rank == 0 and not args.no_mrhs:
        mrhs = mrhs_bench(q, torch, stream, L_MRHS, (4, 8, 16, 32, 48, 64), 10)
    if rank == 0 and not args.no_mrhs and not args.no_solve:
        q.release_work()
        batching = batching_bench(q, L_MRHS, KAPPA, args.big_batch_rhs)
        q.release_work()
    if rank == 0 and not args.no_solve:
        precision = precision_bench(q, L_PREC, KAPPA_PREC, args.batch_rhs, args.batch_slots)
    serving32 = None
    if rank == 0 and not args.no_serve:
        serving = serving_bench(q, args.serve_seconds, args.serve_rate, args.serve_slots, args.serve_budget_gb)
        # the same stream on the 32^3 x 64 gauge field alone (the volume of the solve summary)
        serving32 = serving_bench(q, args.serve32_seconds, args.serve32_rate, args.serve_slots, args.serve_budget_gb,
                                  weights=(0, 0, 0, 1))
    ceiling = compute_ceiling(q, V, ms_native, ms_df64, clocks["sm_mhz"] if clocks else None) if rank == 0 else None
    if rank != 0:
        return None
    peaks = measured_peaks()
    gbs_job = replica_throughput(V * bps, ms_max, world)
    achieved_1 = V * bps / (best_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": gbs_job, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if arith == "f64" else "f64 storage, df64 arithmetic",
        "data": "synthetic (seeded SU(3) links exp(i eps H), plaquette %.4f; Gaussian spinor)" % plaq,
        "config": {"workload": "FP64 Wilson-Dirac apply D psi, 24^3x48, kappa 0.150, theta_t = pi, 18-real links",
                   "lattice_txyz": list(L_BENCH), "sites": V, "bytes_per_site": bps, "flops_per_site": FLOPS_PER_SITE,
                   "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (working set %d MB vs 129 MB)" % (V * bps // 2**20)},
        "gflops": V * FLOPS_PER_SITE / (ms_max * 1e-3) / 1e9 * world,
        "roofline": {"bound": "hbm", "achieved": achieved_1, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved_1 / peaks["hbm_gbs"], "peak_source": peaks["src"],
                     "traffic": profile_traffic("dslash_df64_24x24x24x48.md" if arith == "df64" else
                                                "dslash_f64_24x24x24x48.md"),
                     "traffic_source": "profiles/ ncu capture of the same kernel and lattice (dram read + write)",
                     "compute_ceiling": ceiling},
        "kernels_ms": {"f64": ms_native, "df64": ms_df64},
        "e2e": {"value": V * bps / (ms_e2e * 1e-3) / 1e9 * world, "unit": "GB/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "qcd_applyWilsonTMOp on page-locked host qcd_vector buffers, resident gauge; slab-wise "
                        "copies in and out overlapped with the operator"},
        "gpu_launches": launches,
        "clocks": clocks,
        "solve": solve,
        "precision_32x64": precision,
        "mrhs_operator": mrhs,
        "batching_48x96": batching,
        "serving": serving,
    }
    # the conventional count (8 neighbour spinors + 8 links + out), not the roofline basis
    eff = 8 * 192 + 8 * 144 + 192
    line["effective_bytes"] = {"bytes_per_site": eff, "GB/s": V * eff / (best_ms * 1e-3) / 1e9,
                               "note": "8 neighbour spinors + 8 links + output per site; not the roofline basis"}
    line["serving_32x64"] = serving32
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds, 1)
        if not args.no_solve:
            line["config1_8x16"] = config1_solves(q, args.cpu_seconds / 2)
    line["solve_summary_32x64"] = solve_summary(precision, serving32)
    return line


def solve_summary(precision, serving32):
    """the solve comparison at 32^3 x 64, kappa 0.155, true residual 1e-10
    (last key of the line): RHS-solves/s of the plain FP64 GPU solve (the
    drop-in), of the batched and the single even/odd mixed-precision solves
    and of the served stream on that volume, their ratios to the plain solve
    (target 4), and the served p50 / p99 latency. The served requests draw
    kappa from [0.14, 0.155], where this ensemble's solves take more
    iterations than at 0.155, so the iteration rates (RHS-iterations per
    second) compare the served stream with the single solve as well"""
    if not precision:
        return None
    base = precision["fp64_cgnr"]["rhs_solves_per_s"]
    ns = {"lattice_txyz": precision["lattice_txyz"], "kappa": precision["kappa"], "tol": 1e-10, "target_ratio": 4.0,
          "plain_fp64": base, "single_eo_f16": precision["eo_cgnr_f16"]["rhs_solves_per_s"],
          "batched_eo": precision["batched_mrhs_eo"]["rhs_solves_per_s"],
          "served": serving32["rhs_solves_per_s"] if serving32 else None,
          "served_p50_s": serving32["p50_s"] if serving32 else None,
          "served_p99_s": serving32["p99_s"] if serving32 else None,
          "served_tols": "1e-8 or 1e-10 per request" if serving32 else None,
          "single_eo_f16_iters": precision["eo_cgnr_f16"]["iters"],
          "served_mean_iters_per_rhs": serving32.get("mean_iters_per_rhs") if serving32 else None}
    se = precision["eo_cgnr_f16"]
    ns["single_eo_f16_iterations_per_s"] = se["iters"] * se["rhs_solves_per_s"] if se["rhs_solves_per_s"] else None
    ns["served_iterations_per_s"] = serving32.get("rhs_iterations_per_s") if serving32 else None
    for k in ("single_eo_f16", "batched_eo", "served"):
        ns["ratio_" + k] = ns[k] / base if base and ns[k] else None
    return ns


def run_only(args):
    """one operator variant on the bench lattice, nothing else (profiling target)"""
    import torch

    import qcd_gb300 as q

    if args.only == "serve":
        # arrival-rate sweep of the serving stream (one line per rate)
        rates = [float(r) for r in args.serve_sweep.split(",")]
        return {"only": "serve", "sweep": [serving_bench(q, args.serve_seconds, r, args.serve_slots,
                                                         args.serve_budget_gb) for r in rates]}
    if args.only == "solve":
        # one point-source column solved to 1e-10 (even/odd CGNR, FP16 inner)
        g = q.Gauge(L_BENCH, THETA).synthetic(1000, EPS_PLAQ_060)
        b, x = q.Field(L_BENCH).point((0, 0, 0, 0), 0, 0), q.Field(L_BENCH)
        q.sync()
        t0 = time.perf_counter()
        p = q.solve(x, b, g, KAPPA, 0.0, solver=q.SOLVER_CGNR_EO, inner_prec=q.F16, tol=1e-10, maxiter=args.steps)
        q.sync()
        return {"only": "solve", "s": time.perf_counter() - t0, "iters": p.iters, "status": p.status,
                "true_residual": p.true_residual}
    if args.only == "batch":
        # batched multi-RHS solve of point-source columns on the bench lattice
        g = q.Gauge(L_BENCH, THETA).synthetic(1000, EPS_PLAQ_060)
        n = args.mrhs_n
        srcs = [q.Field(L_BENCH).point((0, 0, 0, 0), c % 12 // 3, c % 3) for c in range(n)]
        xs = [q.Field(L_BENCH) for _ in range(n)]
        batch = q.Batch(g, n, eo=args.eo)
        q.sync()
        t0 = time.perf_counter()
        for c in range(n):
            batch.add(xs[c], srcs[c], KAPPA, 0.0, q.OP_D, tol=1e-10, maxiter=args.steps, tag=c)
        done = []
        while batch.active:
            batch.step(16)
            done += batch.poll()
        q.sync()
        dt = time.perf_counter() - t0
        return {"only": "batch", "rhs": n, "wall_s": dt, "rhs_solves_per_s": n / dt,
                "iters": max(d[2] for d in done), "status": sorted({d[1] for d in done}),
                "max_true_residual": max(d[3] for d in done), "tuned": q.mrhs_tuned(L_BENCH, n)}
    if args.only == "mrhs":
        stream = torch.cuda.current_stream()
        q.set_stream(stream.cuda_stream)
        q.set_mrhs_variant(args.mrhs_variant)
        res = mrhs_bench(q, torch, stream, L_BENCH, (args.mrhs_n,), args.steps)
        return {"only": "mrhs", "variant": args.mrhs_variant, **res["sweep"][0]}
    prec = {"f64": q.F64, "df64": q.F64, "f32": q.F32, "f16": q.F16}[args.only]
    arith = q.ARITH_DF64 if args.only == "df64" else q.ARITH_F64
    g64 = q.Gauge(L_BENCH, THETA).synthetic(1000, EPS_PLAQ_060)
    g = g64 if prec == q.F64 else q.Gauge(L_BENCH, THETA, prec).convert_from(g64)
    f64 = q.Field(L_BENCH).gaussian(2000)
    fin = f64 if prec == q.F64 else q.Field(L_BENCH, prec).copy_from(f64)
    fout = q.Field(L_BENCH, prec)
    stream = torch.cuda.current_stream()
    q.set_stream(stream.cuda_stream)
    ms, n = time_dslash(q, torch, fout, fin, g, args.steps, args.warmup, arith, stream)
    V = L_BENCH[0] * L_BENCH[1] * L_BENCH[2] * L_BENCH[3]
    bps = bytes_per_site(prec, 18 if prec == q.F64 else 12)
    return {"only": args.only, "ms_per_apply": ms, "gbs": V * bps / (ms * 1e-3) / 1e9, "bytes_per_site": bps,
            "launches": n}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    ncores = os.cpu_count() or 1
    cb = cpu_baseline(args.ref_seconds, ncores)
    V = L_BENCH[0] * L_BENCH[1] * L_BENCH[2] * L_BENCH[3]
    ms = 1e3 / cb["applies_per_s"]
    return {"metric": METRIC, "value": cb["value"], "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "FP64 Wilson-Dirac apply D psi, 24^3x48, kappa 0.150, theta_t = pi",
                       "lattice_txyz": list(L_BENCH), "sites": V, "bytes_per_site": bytes_per_site(0, 18),
                       "parallelism": f"{ncores} CPU processes, one apply stream each"},
            "impl": "reference", "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--solve-rhs", type=int, default=4)
    ap.add_argument("--no-mrhs", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--batch-rhs", type=int, default=48, help="point-source columns of the batched 32^3x64 solve")
    ap.add_argument("--batch-slots", type=int, default=48)
    ap.add_argument("--big-batch-rhs", type=int, default=96,
                    help="point-source columns of the 48^3x96 batch (8 positions x 12 columns)")
    ap.add_argument("--serve-seconds", type=float, default=30.0)
    ap.add_argument("--serve-rate", type=float, default=2.0, help="request arrivals per second")
    ap.add_argument("--serve-slots", type=int, default=32)
    ap.add_argument("--serve-budget-gb", type=float, default=120.0)
    ap.add_argument("--serve32-seconds", type=float, default=15.0, help="arrival window of the 32^3x64-only stream")
    ap.add_argument("--serve32-rate", type=float, default=1.0, help="arrivals per second of the 32^3x64-only stream")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=20.0)
    ap.add_argument("--mrhs-n", type=int, default=16, help="--only mrhs / batch: RHS per block / batch slots")
    ap.add_argument("--eo", action="store_true", help="--only batch: even/odd preconditioned batch")
    ap.add_argument("--mrhs-variant", type=int, default=-1,
                    help="--only mrhs: -1 tuned, 1 tensor cores, 64/128/256 SIMT block size")
    ap.add_argument("--serve-sweep", default="0.5,1,2,4", help="--only serve: arrival rates (requests/s)")
    ap.add_argument("--only", choices=["f64", "df64", "f32", "f16", "mrhs", "batch", "solve", "serve"],
                    help="profiling target: time only this operator variant (a few launches under ncu)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.only:
        print(json.dumps(run_only(args)), flush=True)
        return
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        if world > 1:
            import torch

            torch.distributed.init_process_group("nccl")
        line = run_ours(args, rank, world, local_rank)
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
