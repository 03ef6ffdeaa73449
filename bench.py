#!/usr/bin/env python
"""Benchmark of the normal-equations hot path on GB300.

Headline (one JSON line on stdout): the isolated product (A D^-1 A^T) v on
the 100,000 x 400,000 LP (8 nonzeros per column, 3.2M nonzeros) with d
log-uniform in [1e-8, 1e8] -- the SpMV GB/s metric -- in FP64 (the drop-in
precision).  One step = one product = two CSR row-gather passes,
t = B^T v then y = B t with B = A D^-1/2.  Inputs are resident in HBM; L2 is
flushed before every step (a 256 MB write, then a 256 MB read of a second
buffer, so the write's dirty lines are written back before the timed span
rather than during it).  Achieved bandwidth counts the
algorithmic bytes of each pass (values and indices once, both vectors once).

Also reported on the same line: the FP32 product (mixed precision), the
end-to-end product through the C ABI with host buffers, the CPU baseline
(the reference's CSRMV_T / scale / CSRMV_N loops restated in oracle/, one
core), the IPM time to a 1e-8 relative gap on the 2,000 x 6,000 LP (GPU,
plain FP64 PCG, the mixed form against it with the FP64 residual of every
Newton solve, and the direct form with every row a pivot), the learned
part's ablation on held-out multicommodity-flow
LPs and its MLP's forward / training rates, PCG iterations per second (configs 0, 1 and 4 by default), the same
product on the 104M-nonzero block-angular LP, the live
roofline of the dominant kernel and the SM clocks sampled during the timed
region.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference] [--no-ipm] [--no-large]
                    [--pcg-configs 0,1] [--pcg-iters I] [--pcg-only] [--mlp-only [--mlp-rows R]] [--large-only]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "SpMV HBM GB/s: (A D^-1 A^T) v, two CSR row-gather passes (IPM time to 1e-8 gap reported alongside)"
WORKLOAD = "config 1: m=100000 n=400000, 8 nnz/col (3.2M nnz), d log-uniform [1e-8,1e8]"
L2_NOTE = ("flushed before every step: 256 MB write, then 256 MB read of a second buffer (the write's "
           "dirty lines written back before the timed span)")


def alg_bytes(m: int, n: int, nnz: int, elem: int) -> dict:
    """Algorithmic bytes of each pass: values + int32 indices once, row
    pointers once, the gathered vector once, the result once."""
    bt = (elem + 4) * nnz + 4 * (n + 1) + elem * m + elem * n   # t = B^T v (rows of A^T = columns)
    b = (elem + 4) * nnz + 4 * (m + 1) + elem * n + elem * m    # y = B t
    return {"BT": bt, "B": b, "step": bt + b}


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops", 1900.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def gather_bound(nnz: int, pass_ms: float, dev, clocks: dict | None) -> dict:
    """The pass's practical bound for random sparsity: each nonzero gathers an
    entry of a vector that L1 does not hold, i.e. one L1 -> L2 request, and
    an SM's L1 issues at most one such request per clock (profiles/
    spmv_adat_config1.md: that interface is the busiest unit).  bound_us =
    nnz / (SMs x SM clock); frac = bound / measured pass time."""
    import torch

    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    bound_us = nnz / (sms * mhz * 1e6) * 1e6
    return {"requests": int(nnz), "sms": sms, "sm_mhz": mhz, "bound_us": round(bound_us, 2),
            "measured_us": round(pass_ms * 1e3, 2), "frac": round(bound_us / (pass_ms * 1e3), 3)}


def ncu_traffic() -> dict | None:
    p = os.path.join(ROOT, "profiles", "spmv_adat_config1_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
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
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_value(step_ms: float, bytes_per_step: int, ws: int, dev) -> tuple[float, float]:
    """Replicas (one independent product per rank): the slowest rank's step
    time, and the bytes of all ranks over it in GB/s."""
    if ws > 1:
        import torch

        tt = torch.tensor([step_ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(tt.item())
    return step_ms, ws * bytes_per_step / (step_ms * 1e-3) / 1e9


def cpu_adat_baseline(lp, d, seconds: float = 10.0) -> dict:
    """The reference's own loops for one (A D^-1 A^T) v (PCG.cpp:346-358 with
    CSRMV_T / CSRMV_N of Helper.cpp:57-81), restated in oracle/, one core."""
    from oracle import bindings as ob

    rp, ci, v = lp.csr()
    x = np.random.default_rng(1).standard_normal(lp.m)
    nb = alg_bytes(lp.m, lp.n, lp.nnz, 8)["step"] + 8 * lp.n  # + reading d in the scale loop
    reps, t0 = 0, time.perf_counter()
    while True:
        t = ob.csrmv_t(rp, ci, v, x, lp.m, lp.n)
        t /= d
        ob.csrmv_n(rp, ci, v, t, lp.m, lp.n)
        reps += 1
        el = time.perf_counter() - t0
        if el > seconds or reps >= 1000:
            break
    return {"value": nb * reps / el / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
            "sample": "%d products (A D^-1 A^T) v on %s, single thread (the reference's loops are serial)" % (reps, WORKLOAD),
            "seconds": el}


def ipm_run(config: int, precision: str, pivots: int | None = None, lp=None, cg_path: str = "auto",
            oracle: bool = False) -> dict:
    """HSD IPM (the reference's HSD_Main restated) to a 1e-8 gap on the GPU
    backend, with the FP64 residual ||rhs - G x_2|| / ||rhs|| of every Newton
    solve read back after the solve.  oracle: every Newton system of the run
    (d, b_1, b_2 and the solution) is recorded, and after the timed run each
    is solved again on the host in FP64 (cpu_fp64_newton_errors) to report
    the solutions' errors against it."""
    import ctypes as C

    from help_gb300 import backend, hsd, native, lp as L

    name = None
    if lp is None:
        lp = L.make_lp(config, 0)
        k = L.config_pivots(config) if pivots is None else min(pivots, lp.m)
    else:
        name, lp = lp
        k = min(pivots, lp.m)
    solves = []
    recorded = []  # (d, b1, b2, x1, x2) of every Newton solve, when oracle
    m_, n_ = lp.m, lp.n

    def host(ptr, count):
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double)), (count,)).copy()

    with backend.GpuNormalEquations(pivots=k, precision=precision, cg_tol=1e-10, ir_tol=1e-10,
                                    cg_max_iter=1_000_000, cg_path=cg_path) as g:
        lib, ctx = g.lib, g.ctx

        def solve(_c, d, b1, b2, x1, x2):
            rc = lib.help_pcg_solve(ctx, d, b1, b2, x1, x2)
            st = g.stats()
            solves.append((st["rel_residual"], st["fell_back"], st["cg_iterations"], st["cg_iterations_fp32"]))
            if oracle:
                recorded.append((host(d, n_), host(b1, n_), host(b2, m_), host(x1, n_), host(x2, m_)))
            return rc

        fns = (native.CONSTRUCT_FN(lambda _c, m, n, cp, ri, v: lib.help_pcg_construct(ctx, m, n, cp, ri, v)),
               native.RENEW_FN(lambda _c, d: lib.help_pcg_renew(ctx, d)), native.SOLVE_FN(solve),
               native.DESTRUCT_FN(lambda _c: lib.help_pcg_destruct(ctx)),
               native.MATVEC_FN(lambda _c, t, s, v, dest: lib.help_pcg_matvec_acc(ctx, t, s, v, dest)))
        f = lambda fn: C.cast(fn, C.c_void_p).value
        be = native.NeBackend(ctx=None, construct=f(fns[0]), renew=f(fns[1]), solve=f(fns[2]), destruct=f(fns[3]),
                              matvec=f(fns[4]))
        t0 = time.perf_counter()
        r = hsd.solve_lp(lp, be)
        wall = time.perf_counter() - t0
        st = g.stats()
    errs = None
    if oracle and recorded:
        errs = cpu_fp64_newton_errors(lp, recorded)
    res = np.array([s_[0] for s_ in solves]) if solves else np.zeros(1)
    return {"config": "%s: m=%d n=%d nnz=%d" % (name or "config %d" % config, lp.m, lp.n, lp.nnz),
            "form": "%s PCG, k=%d, tol 1e-10, CG path %s" % (
                "plain FP64" if precision == "fp64" else "FP32 CG in FP64 refinement", k,
                {1: "graph", 2: "single cluster", 3: "resident cluster"}.get(int(st["cg_path_used"]), "?")),
            "seconds": round(wall, 3), "status": r["status"], "iterations": r["iterations"],
            "rel_gap": r["rel_gap"], "primal_obj": r["primal_obj"], "primal_infeas": r["primal_infeas"],
            "dual_infeas": r["dual_infeas"], "cg_iterations": int(st["cg_iterations_total"]),
            "cg_iterations_fp32": int(sum(s_[3] for s_ in solves)), "solves": len(solves),
            "solves_finished_in_fp64": int(sum(s_[1] for s_ in solves)),
            "newton_residual_max": float(res.max()), "newton_residual_median": float(np.median(res)),
            "backend_seconds": round(r["backend_s"], 3),
            **({"newton_solution_errors": errs} if errs else {})}


def cpu_fp64_newton_errors(lp, recorded) -> dict:
    """Each recorded Newton system [D A^T; A 0][x1; x2] = [b1; b2] solved
    again on the host, independently of the GPU library: dense
    G = A D^-1 A^T, LAPACK Cholesky (scipy; where G is not
    numerically positive definite: LU), one step of iterative refinement, then
    x1 = D^-1 (b1 - A^T x2) (UsePCG_CPU.cpp:103-177's reduction).  Returns
    the relative errors of the GPU's x1, x2 against it."""
    import scipy.linalg as sl

    A = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        A[lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]], j] = lp.val[lp.col_ptr[j]:lp.col_ptr[j + 1]]
    ex, ey, n_lu = [], [], 0
    last_d, fac = None, None
    for d, b1, b2, x1, x2 in recorded:
        if last_d is None or not np.array_equal(d, last_d):
            G = (A / d) @ A.T
            try:
                fac = ("chol", sl.cho_factor(G, lower=True))
            except np.linalg.LinAlgError:
                fac = ("lu", sl.lu_factor(G))
                n_lu += 1
            last_d = d
        solve = (lambda r: sl.cho_solve(fac[1], r)) if fac[0] == "chol" else (lambda r: sl.lu_solve(fac[1], r))
        rhs = A @ (b1 / d) - b2
        ox2 = solve(rhs)
        ox2 += solve(rhs - G @ ox2)
        ox1 = (b1 - A.T @ ox2) / d
        ex.append(float(np.linalg.norm(x1 - ox1) / max(np.linalg.norm(ox1), 1e-300)))
        ey.append(float(np.linalg.norm(x2 - ox2) / max(np.linalg.norm(ox2), 1e-300)))
    return {"oracle": "host FP64: dense A D^-1 A^T, LAPACK Cholesky (scipy; LU where not positive definite: %d "
                      "renews), one refinement step; independent of the GPU library" % n_lu,
            "dy_rel_err_max": max(ey), "dy_rel_err_median": float(np.median(ey)),
            "dx_rel_err_max": max(ex), "dx_rel_err_median": float(np.median(ex))}


def ipm_time(config: int = 0) -> dict:
    """Plain FP64 IPM time, and the mixed form measured against it."""
    plain = ipm_run(config, "fp64", oracle=True)
    mixed = ipm_run(config, "mixed", oracle=True)
    mixed["obj_rel_diff_vs_fp64"] = abs(mixed["primal_obj"] - plain["primal_obj"]) / abs(plain["primal_obj"])
    plain["mixed"] = mixed
    # direct form: every row a pivot, i.e. the full Cholesky of A D^-1 A^T
    direct = ipm_run(config, "fp64", pivots=1 << 30)
    direct["obj_rel_diff_vs_fp64"] = abs(direct["primal_obj"] - plain["primal_obj"]) / abs(plain["primal_obj"])
    plain["direct"] = direct
    # the multicommodity-flow family of config 3 at a size whose IPM finishes
    # in seconds (24 x 24 grid, 4 commodities): the auto CG path (resident
    # cluster) against the whole-GPU graph
    from help_gb300 import lp as L
    mcf = ("multicommodity flow 24 x 24 grid, 4 commodities (config 3's generator)",
           L.generate(L.spec_mcf(24, 4, 3), 11))
    m_auto = ipm_run(0, "fp64", pivots=16, lp=mcf)
    m_graph = ipm_run(0, "fp64", pivots=16, lp=mcf, cg_path="graph")
    plain["mcf"] = {"auto": m_auto, "graph": m_graph, "paired": ipm_paired(mcf[1], 16, m_auto, mcf[0])}
    plain["paired"] = ipm_paired(L.make_lp(config, 0), L.config_pivots(config), plain, "config %d" % config)
    return plain


def ipm_paired(lp, k: int, single: dict, name: str) -> dict:
    """The same plain FP64 IPM with the bottom system and the first search
    direction of every iteration solved at once on two contexts (backend
    solve2, help_pcg_pair); the run is bitwise the single context's."""
    from help_gb300 import backend, hsd

    with backend.GpuPairNormalEquations(pivots=min(k, lp.m), precision="fp64", cg_tol=1e-10, ir_tol=1e-10,
                                        cg_max_iter=1_000_000) as p:
        t0 = time.perf_counter()
        r = hsd.solve_lp(lp, p.ne_backend())
        wall = time.perf_counter() - t0
        s0, s1 = p.stats(0), p.stats(1)
    return {"workload": "%s: m=%d n=%d nnz=%d" % (name, lp.m, lp.n, lp.nnz),
            "form": "plain FP64 PCG, k=%d, bottom system and first direction solved together on two contexts"
                    % min(k, lp.m),
            "seconds": round(wall, 3), "status": r["status"], "iterations": r["iterations"], "rel_gap": r["rel_gap"],
            "primal_obj": r["primal_obj"], "solves": r["solves"],
            "cg_iterations": int(s0["cg_iterations_total"] + s1["cg_iterations_total"]),
            "same_objective_bitwise_as_single": bool(r["primal_obj"] == single["primal_obj"]),
            "speedup_vs_single": round(single["seconds"] / wall, 3) if wall > 0 else None}


def spmv_large(steps: int, warmup: int, local: int) -> dict:
    """(A D^-1 A^T) v on the block-angular LP of 1,924,000 x 8,000,000 with
    ~104M nonzeros (32 blocks + 4,000 linking rows): 2.8 GB of algorithmic
    traffic per FP64 product, where launch costs no longer matter."""
    import torch

    from help_gb300 import backend, lp as L

    lp = L.make_lp(4, 0)
    m, n, nnz = lp.m, lp.n, lp.nnz
    rng = np.random.default_rng(4)
    d = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), n))
    dev = torch.device("cuda", local)
    out = {"workload": "config 4: m=%d n=%d nnz=%d, d log-uniform [1e-8,1e8]" % (m, n, nnz)}
    with backend.GpuNormalEquations(pivots=1, precision="mixed", device=local) as g:
        g.LinearEquation_Construct(lp)
        del lp
        g.RenewLinearEquation(d)
        for prec, dt in (("f64", torch.float64), ("f32", torch.float32)):
            x = torch.randn(m, dtype=dt, device=dev)
            t = torch.empty(n, dtype=dt, device=dev)
            y = torch.empty(m, dtype=dt, device=dev)
            fp32 = prec == "f32"
            evs = []
            for it in range(warmup + steps):
                e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
                e0.record()
                g.matvec_dev("BT", x.data_ptr(), t.data_ptr(), fp32=fp32)
                e1.record()
                g.matvec_dev("B", t.data_ptr(), y.data_ptr(), fp32=fp32)
                e2.record()
                if it >= warmup:
                    evs.append((e0, e1, e2))
            torch.cuda.synchronize()
            ab = alg_bytes(m, n, nnz, 8 if prec == "f64" else 4)
            bt = sum(a.elapsed_time(b) for a, b, _ in evs) / len(evs)
            bb = sum(b.elapsed_time(c) for _, b, c in evs) / len(evs)
            out[prec] = {"value": round(ab["step"] / ((bt + bb) * 1e-3) / 1e9, 1), "unit": "GB/s",
                         "ms_per_step": round(bt + bb, 4),
                         "passes_gbs": {"BT": round(ab["BT"] / (bt * 1e-3) / 1e9, 1),
                                        "B": round(ab["B"] / (bb * 1e-3) / 1e9, 1)},
                         "gather_bound": {"BT": gather_bound(nnz, bt, dev, None),
                                          "B": gather_bound(nnz, bb, dev, None)}}
        # the HSD driver's own products (dest += sign A v, dest += sign A^T y)
        # on the device copy of A, host buffers in and out (help_pcg_matvec_acc)
        from help_gb300 import native
        hp = {}
        for name, tr, nin, nout in (("A_v", 0, n, m), ("AT_y", 1, m, n)):
            v = rng.standard_normal(nin)
            dest = rng.standard_normal(nout)
            times = []
            for it in range(4):
                t0 = time.perf_counter()
                rc = g.lib.help_pcg_matvec_acc(g.ctx, tr, -1, native.ptr(v), native.ptr(dest))
                times.append(time.perf_counter() - t0)
                assert rc == native.HELP_OK
            hp[name + "_ms"] = round(1e3 * float(np.median(times[1:])), 2)
        out["hsd_products"] = dict(hp, note="wall time per call through the C ABI with host buffers (v and "
                                            "dest read from the host arrays, one SpMV pass storing into dest), "
                                            "median of 3 after 1 warm-up")
    return out


def pcg_rate(config: int, iters: int, local: int, k: int | None = None) -> dict:
    """PCG iterations per second on the given configuration with its pivot
    count (or k), d log-uniform in [1e-8, 1e8]: one CG run of exactly `iters`
    iterations (unreachable tolerance) in FP64 and one in FP32 (the mixed
    form's inner solver), timed on the device with CUDA events."""
    from help_gb300 import backend, lp as L

    lp = L.make_lp(config, 0)
    rng = np.random.default_rng(7)
    d = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), lp.n))
    b = rng.standard_normal(lp.m)
    k = L.config_pivots(config) if k is None else k
    out = {}
    with backend.GpuNormalEquations(pivots=k, precision="mixed", cg_tol=1e-300, cg_max_iter=iters,
                                    device=local) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        renew_ms = g.stats()["renew_ms"]
        for prec in ("f64", "f32"):
            g.cg(b, fp32=prec == "f32")  # graph capture and warm-up
            _, it = g.cg(b, fp32=prec == "f32")
            st = g.stats()
            us = st["cg_kernel_ms"] * 1e3 / max(it, 1)
            out[prec] = {"iterations": int(it), "us_per_iteration": round(us, 2), "iterations_per_s": round(1e6 / us, 1)}
    out.update({"workload": "config %d: m=%d n=%d nnz=%d, k=%d, nnz(C)=%d" % (config, lp.m, lp.n, lp.nnz, k, st["nnz_c"]),
                "renew_ms": round(renew_ms, 2),
                "path": {1: "graph", 2: "single cluster", 3: "resident cluster"}.get(int(st["cg_path_used"]), "?")})
    return out


def cpu_pcg_rate(config: int, k: int, iters: int) -> dict:
    """The reference's CG loop (PCG.cpp:296-395 with its partial-Cholesky
    preconditioner, greedy pivots, PCG.cpp:38-196) restated in oracle/, one
    core (the reference's PCG path is serial): `iters` iterations at an
    unreachable tolerance on the same system as pcg_rate, the factor build
    timed apart."""
    from help_gb300 import lp as L
    from oracle import bindings as ob

    lp = L.make_lp(config, 0)
    rng = np.random.default_rng(7)
    d = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), lp.n))
    b = rng.standard_normal(lp.m)
    rp, ci, v = lp.csr()
    t0 = time.perf_counter()
    pc = ob.PartialCholesky(rp, ci, v, d, lp.m, lp.n, k)
    build = time.perf_counter() - t0
    del pc
    t0 = time.perf_counter()
    _, it = ob.pcg(rp, ci, v, d, b, lp.m, lp.n, k, tol=1e-300, max_iter=iters)
    tot = time.perf_counter() - t0
    us = (tot - build) * 1e6 / max(it, 1)
    return {"workload": "config %d: m=%d n=%d nnz=%d, k=%d" % (config, lp.m, lp.n, lp.nnz, k), "cores": 1,
            "kind": "port", "iterations": int(it), "us_per_iteration": round(us, 1),
            "iterations_per_s": round(1e6 / us, 1), "factor_build_s": round(build, 3)}


def adat_assembly(config: int, local: int, threads: int) -> dict:
    """The explicit upper triangle of A D^-1 A^T: the reference's
    ADAt_Allocate (symbolic, serial) + ADAt_Calc (numeric, its OpenMP row
    loop; Helper.cpp:215-377) restated in oracle/ on `threads` host cores,
    beside the GPU assembly (help_adat_assemble: count pass, fill pass,
    result copied to host arrays; wall time of the second of two calls),
    checked equal bit for bit."""
    from help_gb300 import backend, lp as L
    from oracle import bindings as ob

    lp = L.make_lp(config, 0)
    rng = np.random.default_rng(3)
    w = 1.0 / np.exp(rng.uniform(np.log(1e-8), np.log(1e8), lp.n))
    rp, ci, v = lp.csr()
    cpu = ob.adat_timed(rp, ci, v, lp.col_ptr, lp.row_ind, lp.val, w, lp.m, lp.n, threads)
    with backend.GpuNormalEquations(pivots=1, device=local) as g:
        g.LinearEquation_Construct(lp)
        g.adat(w)
        t0 = time.perf_counter()
        grp, gcol, gval = g.adat(w)
        gs = time.perf_counter() - t0
    orp, ocol, oval = ob.adat(rp, ci, v, lp.col_ptr, lp.row_ind, lp.val, w, lp.m, lp.n)
    same = bool(np.array_equal(grp, orp) and np.array_equal(gcol, ocol) and np.array_equal(gval, oval))
    return {"workload": "config %d: m=%d n=%d nnz=%d" % (config, lp.m, lp.n, lp.nnz), "nnz_upper": cpu["nnz"],
            "gpu_s": round(gs, 4), "cpu_numeric_s": round(cpu["numeric_s"], 4),
            "cpu_symbolic_s": round(cpu["symbolic_s"], 4), "cpu_threads": cpu["threads"], "kind": "port",
            "bitwise_equal": same}


def _cpu_ipm_worker(conn, core: int | None) -> None:
    """Spawned process: the HSD driver over the oracle backend (the
    reference's UsePCG_CPU / PCG restated, 10 pivots, CG to 1e-10 as the GPU
    runs) on the 2,000 x 6,000 LP, on one host core."""
    try:
        if core is not None and hasattr(os, "sched_setaffinity"):
            os.sched_setaffinity(0, {core})
        from help_gb300 import hsd, lp as L
        from oracle import bindings as ob

        lp = L.make_lp(0, 0)
        ora = ob.OracleNormalEquations(pivots=10, tol=1e-10)
        t0 = time.perf_counter()
        r = hsd.solve_lp(lp, ora.ne_backend())
        el = time.perf_counter() - t0
        conn.send({"seconds": round(el, 2), "status": r["status"], "iterations": r["iterations"],
                   "cg_iterations": ora.total_iters(), "primal_obj": r["primal_obj"], "rel_gap": r["rel_gap"],
                   "cores": 1, "kind": "port", "core": core,
                   "sample": "whole IPM to 1e-8 gap on config 0 (m=2000 n=6000), 10 pivots, CG tol 1e-10"})
    except Exception as e:  # reported, not fatal
        conn.send({"error": str(e)})
    conn.close()


def start_cpu_ipm():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    parent, child = ctx.Pipe(duplex=False)
    cores = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else []
    core = cores[-1] if len(cores) > 2 else None
    p = ctx.Process(target=_cpu_ipm_worker, args=(child, core), daemon=True)
    p.start()
    child.close()
    if core is not None:
        # keep this process (and the CPU baselines it times) off that core
        os.sched_setaffinity(0, set(cores) - {core})
    return p, parent


def finish_cpu_ipm(handle, timeout: float = 600.0) -> dict:
    p, conn = handle
    out = conn.recv() if conn.poll(timeout) else {"error": "did not finish within %.0f s" % timeout}
    p.join(5)
    return out


def ipm_large(params, local: int, caps: dict) -> dict:
    """The interior-point method on the large configurations, plain FP64 PCG
    against the learned + mixed form (FP32 CG in FP64 refinement with the
    trained model attached), each under the same wall-clock cap: gap,
    infeasibilities and CG iterations against time at every iteration, and
    the time to a 1e-8 gap where one is reached.  Solves stop at 20,000 CG
    iterations and hand back their inexact direction (cap_ok)."""
    from help_gb300 import learned, lp as L

    out = {}
    for config, cap in caps.items():
        lp = L.make_lp(config, 0)
        k = L.config_pivots(config)
        res = {"workload": "config %d: m=%d n=%d nnz=%d, k=%d" % (config, lp.m, lp.n, lp.nnz, k),
               "cap_s": cap}
        for arm, prm, prec in (("plain_fp64", None, "fp64"), ("learned_mixed", params, "mixed")):
            try:
                r = learned.evaluate(lp, k, prm, cg_tol=1e-10, device=local, precision=prec, max_seconds=cap,
                                     cg_max_iter=20000, cap_ok=True, trace=True)
                r["seconds"] = round(r["seconds"], 2)
                r["time_to_1e-8_s"] = r["seconds"] if r["status"] == 0 and r["rel_gap"] <= 1e-8 else None
                res[arm] = r
            except Exception as e:
                res[arm] = {"error": str(e)}
        if config == 1:
            # both arms again with the bottom system and first direction of
            # each iteration solved together on two contexts (help_pcg_pair)
            for arm, prm, prec in (("plain_fp64_paired", None, "fp64"), ("learned_mixed_paired", params, "mixed")):
                try:
                    r = learned.evaluate(lp, k, prm, cg_tol=1e-10, device=local, precision=prec, max_seconds=cap,
                                         cg_max_iter=20000, cap_ok=True, trace=True, paired=True)
                    r["seconds"] = round(r["seconds"], 2)
                    r["time_to_1e-8_s"] = r["seconds"] if r["status"] == 0 and r["rel_gap"] <= 1e-8 else None
                    res[arm] = r
                except Exception as e:
                    res[arm] = {"error": str(e)}
        out["config%d" % config] = res
        del lp
    return out


def learned_ablation() -> dict:
    """The learned warm start / Schur-diagonal correction trained on the IPM
    iterates of 6 seeded multicommodity-flow LPs (8 x 8 grid, 3 commodities),
    measured on 4 held-out seeds against the plain FP64 PCG and against the
    same warm start without the network (scale 1, no diagonal correction)."""
    from help_gb300 import learned, lp as L

    spec = dict(grid=8, commodities=3, pairs=3)
    data = [learned.targets(lp, learned.collect(lp, 16)) for lp in (L.generate(L.spec_mcf(**spec), s) for s in range(6))]
    train = {k: np.concatenate([d[k] for d in data]) for k in ("X", "T", "W")}
    t0 = time.perf_counter()
    params, losses = learned.train(train, steps=400)
    train_s = time.perf_counter() - t0
    runs = []
    for s in (100, 101, 102, 103):
        lp = L.generate(L.spec_mcf(**spec), s)
        a, b = learned.evaluate(lp, 16, None), learned.evaluate(lp, 16, params)
        c = learned.evaluate(lp, 16, learned.fixed_warm_params())
        dh = learned.evaluate(lp, 16, learned.diag_head_only(params))
        wh = learned.evaluate(lp, 16, learned.warm_head_only(params))
        lm = learned.evaluate(lp, 16, params, precision="mixed")  # learned + mixed, the benchmark's chosen form
        runs.append({"seed": s, "cg_plain": a["cg_iterations"], "cg_learned": b["cg_iterations"],
                     "cg_fixed_warm_start": c["cg_iterations"], "cg_learned_diag_head_only": dh["cg_iterations"],
                     "cg_learned_warm_head_only": wh["cg_iterations"],
                     "cg_learned_mixed": lm["cg_iterations"], "s_learned_mixed": round(lm["seconds"], 3),
                     "obj_rel_diff_learned_mixed": abs(lm["primal_obj"] - a["primal_obj"]) / abs(a["primal_obj"]),
                     "s_plain": round(a["seconds"], 3), "s_learned": round(b["seconds"], 3),
                     "obj_rel_diff": abs(a["primal_obj"] - b["primal_obj"]) / abs(a["primal_obj"]),
                     "fallbacks": b["learned_fallbacks"]})
    return {"train_rows": int(train["X"].shape[0]), "train_steps": 400, "train_seconds": round(train_s, 2),
            "loss_first": losses[0], "loss_last": losses[-1], "held_out": runs}, params


def mlp_rate(rows: int, reps: int, local: int) -> dict:
    """The learned part's MLP (16 -> 64 -> 64 -> 2, BF16 in, FP32 accumulate)
    on `rows` seeded feature rows: the inference forward the solver runs after
    each renew (tcgen05, TMEM accumulators; CUDA events on its stream over
    `reps` launches, inputs resident) and one training step's forward +
    backward (mma.sync, activations stored; host wall time, synchronised).
    Algorithmic FLOPs: 2 (16*64 + 64*64 + 64*2) per row."""
    import torch

    from help_gb300 import learned
    from help_gb300 import native

    rng = np.random.default_rng(1)
    x = rng.standard_normal((rows, native.MLP_IN)).astype(np.float32)
    x[:, 11:] = 0.0
    t = rng.standard_normal((rows, native.MLP_OUT)).astype(np.float32)
    m = learned.Mlp(local, learned.init_params(2))
    try:
        xb = torch.from_numpy(learned.bf16_bits(x).view(np.int16)).cuda(local)
        tt, ww = torch.from_numpy(t).cuda(local), torch.ones((rows, native.MLP_OUT), dtype=torch.float32, device=xb.device)
        out = torch.empty((rows, native.MLP_OUT), dtype=torch.float32, device=xb.device)
        st = torch.cuda.current_stream()
        fwd = lambda: m._check(m.lib.help_mlp_forward(m.h, xb.data_ptr(), rows, out.data_ptr(), st.cuda_stream))
        for _ in range(3):
            fwd()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fwd()
        e1.record(st)
        torch.cuda.synchronize()
        fwd_ms = e0.elapsed_time(e1) / reps
        for _ in range(2):
            m.loss_grad(xb, tt, ww, rows)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            m.loss_grad(xb, tt, ww, rows)
        torch.cuda.synchronize()
        lg_ms = (time.perf_counter() - t0) / 3 * 1e3
    finally:
        m.close()
    flops = 2.0 * rows * (native.MLP_IN * native.MLP_HIDDEN + native.MLP_HIDDEN ** 2 + native.MLP_HIDDEN * native.MLP_OUT)
    pk = peaks()
    tf = flops / fwd_ms / 1e9
    return {"rows": rows, "forward_us": round(fwd_ms * 1e3, 2), "forward_rows_per_s": round(rows / fwd_ms * 1e3),
            "forward_tflops": round(tf, 1), "forward_frac_of_bf16_peak": round(tf / pk["bf16_tflops"], 4),
            "bf16_peak_source": pk["source"],
            "forward_gbs": round(rows * (2 * native.MLP_IN + 4 * native.MLP_OUT) / fwd_ms / 1e6, 1),
            "train_step_ms": round(lg_ms, 3), "forward_kernel": "k_mlp_fwd_tc (tcgen05.mma kind::f16, M=128)",
            "train_kernels": "k_mlp_fwd<true>, k_mlp_bwd (mma.sync m16n8k16)"}


def presolve_time() -> dict:
    """The host dependent-row presolve (help_lp_remove_dependent_rows, one
    thread): the 200 x 200 grid, 8-commodity flow with every node row kept
    (eight rows short of full rank), and the random config-1 matrix, for
    which it reports that it does not apply."""
    from help_gb300 import lp as L

    out = {"cores": 1}
    lp = L.generate(L.spec_mcf(200, 8, grounded=False), 0)
    t = time.perf_counter()
    _, removed = L.remove_dependent_rows(lp)
    out["mcf_200x200x8_ungrounded"] = {"rows": lp.m, "nnz": lp.nnz, "rows_removed": int(removed.sum()),
                                       "s": round(time.perf_counter() - t, 3)}
    lp1 = L.make_lp(1, 0)
    t = time.perf_counter()
    try:
        _, removed = L.remove_dependent_rows(lp1)
        result = "%d rows removed" % int(removed.sum())
    except L.PresolveNotApplicable:
        result = "not applicable (fill past the limits)"
    out["config1_random"] = {"rows": lp1.m, "nnz": lp1.nnz, "result": result,
                             "s": round(time.perf_counter() - t, 3)}
    return out


def numpy_instance(m: int, n: int, per_col: int, seed: int):
    """The configuration's generator recipe in numpy alone (for the reference
    arm, which loads none of this project's libraries): `per_col` distinct
    uniform-random rows per column, values N(0,1); returned as CSR."""
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, m, (n, per_col))
    while True:
        rows.sort(axis=1)
        dup = np.any(rows[:, 1:] == rows[:, :-1], axis=1)
        if not dup.any():
            break
        rows[dup] = rng.integers(0, m, (int(dup.sum()), per_col))
    r = rows.ravel()
    col = np.repeat(np.arange(n), per_col)
    val = rng.standard_normal(r.size)
    order = np.lexsort((col, r))
    rp = np.zeros(m + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=m), out=rp[1:])
    return rp, col[order].astype(np.int32), np.ascontiguousarray(val[order])


def bench_config(ws: int) -> dict:
    return {"workload": WORKLOAD, "l2": L2_NOTE, "parallelism": "replicas" if ws > 1 else "single GPU"}


def run_reference(args) -> None:
    """The reference's own CPU loops for the path (CSRMV_T, the D^-1 scale and
    CSRMV_N, Helper.cpp:57-81, PCG.cpp:346-358; restated in oracle/ -- the
    reference's own build needs its sources, which the GPU host does not
    have) on the same configuration, one core (those loops are serial)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    m, n = 100000, 400000
    rp, ci, v = numpy_instance(m, n, 8, 0)
    rng = np.random.default_rng(0)
    d = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), n))
    from oracle import bindings as ob

    x = rng.standard_normal(m)
    nb = alg_bytes(m, n, len(ci), 8)["step"] + 8 * n
    for _ in range(args.warmup):
        t = ob.csrmv_t(rp, ci, v, x, m, n)
        t /= d
        ob.csrmv_n(rp, ci, v, t, m, n)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        t = ob.csrmv_t(rp, ci, v, x, m, n)
        t /= d
        ob.csrmv_n(rp, ci, v, t, m, n)
        ts.append(time.perf_counter() - t0)
    tot = sum(ts)
    val = nb * len(ts) / tot / 1e9
    out = {"metric": METRIC, "value": round(val, 3), "unit": "GB/s", "impl": "reference", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * tot / len(ts), 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": bench_config(ws),
           "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": 1, "kind": "port",
                            "sample": "%d products on the configuration's recipe generated in numpy; the "
                                      "reference's CSRMV_T, scale, CSRMV_N loops restated in oracle/ (the "
                                      "reference's own build needs its sources, absent on this host)" % len(ts)},
           "e2e": {"value": round(val, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-ipm", action="store_true", help="skip the IPM-time and learned-part measurements")
    ap.add_argument("--no-large", action="store_true", help="skip the 104M-nonzero SpMV measurement")
    ap.add_argument("--pcg-configs", default="0,1,4", help="configurations whose PCG iteration rate is measured")
    ap.add_argument("--pcg-iters", type=int, default=500, help="CG iterations per rate measurement")
    ap.add_argument("--pcg-only", action="store_true", help="only the PCG iteration rates (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines beyond the product loop")
    ap.add_argument("--no-ipm-large", action="store_true", help="skip the capped IPM runs on configs 1 and 4")
    ap.add_argument("--ipm-large-caps", default="1:25,4:45", help="config:seconds per arm of the capped IPM runs")
    ap.add_argument("--mlp-only", action="store_true", help="only the learned part's MLP rates (profiling runs)")
    ap.add_argument("--large-only", action="store_true", help="only the 104M-nonzero product (profiling runs)")
    ap.add_argument("--mlp-rows", type=int, default=2_000_000, help="feature rows of the MLP rate measurement")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.pcg_only:
        import torch

        ws, rank, local = dist_env()
        torch.cuda.set_device(local)
        out = {c: pcg_rate(int(c), args.pcg_iters, local) for c in args.pcg_configs.split(",") if c}
        print(json.dumps({"pcg": out}), flush=True)
        return
    if args.large_only:
        import torch

        ws, rank, local = dist_env()
        torch.cuda.set_device(local)
        print(json.dumps({"spmv_large": spmv_large(max(1, args.steps), max(1, args.warmup), local)}), flush=True)
        return
    if args.mlp_only:
        import torch

        ws, rank, local = dist_env()
        torch.cuda.set_device(local)
        print(json.dumps({"mlp": mlp_rate(args.mlp_rows, max(1, args.steps), local)}), flush=True)
        return

    ws, rank, local = dist_env()
    cpu_ipm = start_cpu_ipm() if rank == 0 and not args.no_cpu and not args.no_ipm else None

    import torch

    from help_gb300 import backend, lp as L

    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    lp = L.make_lp(1, 0)
    m, n, nnz = lp.m, lp.n, lp.nnz
    rng = np.random.default_rng(0)
    d = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), n))
    g = backend.GpuNormalEquations(pivots=L.config_pivots(1), precision="mixed", device=local)
    g.LinearEquation_Construct(lp)
    g.RenewLinearEquation(d)

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    flush_r = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def flush_l2():
        # evict everything with a write, then replace the write's dirty lines
        # by clean ones, so their write-back does not land in the timed kernel
        flush.fill_(1.0)
        flush_r.sum()
    res = {}
    for prec, dt in (("f64", torch.float64), ("f32", torch.float32)):
        x = torch.randn(m, dtype=dt, device=dev)
        t = torch.empty(n, dtype=dt, device=dev)
        y = torch.empty(m, dtype=dt, device=dev)
        fp32 = prec == "f32"

        def step(times):
            flush_l2()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            g.matvec_dev("BT", x.data_ptr(), t.data_ptr(), fp32=fp32)
            e1.record()
            g.matvec_dev("B", t.data_ptr(), y.data_ptr(), fp32=fp32)
            e2.record()
            if times is not None:
                times.append((e0, e1, e2))

        for _ in range(args.warmup):
            step(None)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if prec == "f64" else None
        if sampler:
            sampler.start()
        evs = []
        for _ in range(args.steps):
            step(evs)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        bt = [a.elapsed_time(b) for a, b, _ in evs]
        bb = [b.elapsed_time(c) for _, b, c in evs]
        tot = [a.elapsed_time(c) for a, _, c in evs]
        res[prec] = {"bt_ms": sum(bt) / len(bt), "b_ms": sum(bb) / len(bb), "step_ms": sum(tot) / len(tot),
                     "clocks": clocks}

    # correctness of the timed product (FP64 vs a direct host recomputation is the parity test's job;
    # here: FP32 and FP64 agree)
    ab64 = alg_bytes(m, n, nnz, 8)
    ab32 = alg_bytes(m, n, nnz, 4)
    step_ms, value = replica_value(res["f64"]["step_ms"], ab64["step"], ws, dev)

    pk = peaks()
    dom = "B" if res["f64"]["b_ms"] >= res["f64"]["bt_ms"] else "BT"
    dom_ms = res["f64"]["b_ms"] if dom == "B" else res["f64"]["bt_ms"]
    achieved = ab64[dom] / (dom_ms * 1e-3) / 1e9
    tr = ncu_traffic()
    roof = {"bound": "hbm", "kernel": "k_spmv<double> pass %s (%s)" % (dom, "y = B t" if dom == "B" else "t = B^T v"),
            "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "peak_source": pk["source"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4), "algorithmic_bytes": ab64[dom],
            "traffic": (tr or {}).get(dom), "traffic_source": (tr or {}).get("source"),
            "gather_bound": gather_bound(nnz, dom_ms, dev, res["f64"]["clocks"])}

    # end to end through the C ABI with host buffers (H2D v, D2H y every step)
    # (help_pcg_matvec: the host vector in, the product out, synchronous); L2
    # is flushed before each step, outside the timed span
    xh = rng.standard_normal(m)
    for _ in range(max(args.warmup, 3)):
        g.matvec("ADAT", xh)
    spans = []
    for _ in range(args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.matvec("ADAT", xh)
        spans.append(time.perf_counter() - t0)
    e2e_s = sum(spans) / len(spans)
    e2e = {"value": round(ab64["step"] / e2e_s / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": 8 * m,
           "d2h_bytes_per_step": 8 * m, "us_per_step": round(e2e_s * 1e6, 1),
           "note": "host wall time of each help_pcg_matvec call (synchronous): the input read from the host "
                           "array by a copy kernel, both passes, a copy kernel writing the host "
                           "output array (Grace: pageable host memory through the host page tables; "
                           "cudaMemcpyAsync copies where the device cannot)"}

    extra = {}
    cpu = None
    params = None
    if rank == 0:
        cpu = cpu_adat_baseline(lp, d, seconds=10.0)
        if not args.no_ipm:
            try:
                extra["ipm"] = ipm_time(0)
            except Exception as e:  # reported, not fatal for the kernel line
                extra["ipm"] = {"error": str(e)}
            try:
                extra["learned"], params = learned_ablation()
            except Exception as e:
                extra["learned"], params = {"error": str(e)}, None
            try:
                extra["mlp"] = mlp_rate(args.mlp_rows, 20, local)
            except Exception as e:
                extra["mlp"] = {"error": str(e)}
            try:
                extra["presolve"] = presolve_time()
            except Exception as e:
                extra["presolve"] = {"error": str(e)}
    g.close()
    if rank == 0:
        extra["pcg"] = {}
        for c in [int(v) for v in args.pcg_configs.split(",") if v]:
            try:
                extra["pcg"]["config%d" % c] = pcg_rate(c, args.pcg_iters, local)
            except Exception as e:
                extra["pcg"]["config%d" % c] = {"error": str(e)}
        if not args.no_cpu:
            # like for like with the reference's shipped pivot count (PCG.h:20)
            try:
                extra["pcg"]["config1_k10"] = pcg_rate(1, args.pcg_iters, local, k=10)
            except Exception as e:
                extra["pcg"]["config1_k10"] = {"error": str(e)}
            cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
            extra["cpu"] = {"host_cores": cores, "pcg_rate": {}}
            for c, it in ((0, 2000), (1, 100)):
                try:
                    extra["cpu"]["pcg_rate"]["config%d_k10" % c] = cpu_pcg_rate(c, 10, it)
                except Exception as e:
                    extra["cpu"]["pcg_rate"]["config%d_k10" % c] = {"error": str(e)}
            extra["adat_assembly"] = {}
            for c in (1, 2):
                try:
                    extra["adat_assembly"]["config%d" % c] = adat_assembly(c, local, max(1, cores - 2))
                except Exception as e:
                    extra["adat_assembly"]["config%d" % c] = {"error": str(e)}
    if rank == 0 and not args.no_large:
        try:
            extra["spmv_large"] = spmv_large(max(3, args.steps // 3), 2, local)
        except Exception as e:
            extra["spmv_large"] = {"error": str(e)}
    if rank == 0 and not args.no_ipm_large:
        caps = {int(a): float(b) for a, b in (kv.split(":") for kv in args.ipm_large_caps.split(",") if kv)}
        try:
            extra["ipm_large"] = ipm_large(params, local, caps)
        except Exception as e:
            extra["ipm_large"] = {"error": str(e)}
    if cpu_ipm is not None:
        extra.setdefault("cpu", {})["ipm_config0"] = finish_cpu_ipm(cpu_ipm)

    if rank == 0:
        out = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(step_ms, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, config 1)",
            "config": bench_config(ws),
            "roofline": roof,
            "fp32": {"value": round(ab32["step"] / (res["f32"]["step_ms"] * 1e-3) / 1e9, 2), "unit": "GB/s",
                     "ms_per_step": round(res["f32"]["step_ms"], 5),
                     "frac": round(ab32["step"] / (res["f32"]["step_ms"] * 1e-3) / 1e9 / pk["hbm_gbs"], 4)},
            "passes_ms": {"f64": {"BT": round(res["f64"]["bt_ms"], 5), "B": round(res["f64"]["b_ms"], 5)},
                          "f32": {"BT": round(res["f32"]["bt_ms"], 5), "B": round(res["f32"]["b_ms"], 5)}},
            "e2e": e2e,
            "cpu_baseline": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in cpu.items()} if cpu else None,
            "gpu_launches": 2 * args.steps,
            "clocks": res["f64"]["clocks"],
        }
        out.update(extra)
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
