"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference's sources are available and oracle/ref's recipe
has built them (oracle/_ref/libhelp_ref.so, oracle/_ref/help_ref):

    make -C oracle/ref && python tests/golden/make_golden.py

Fixtures (all instances come from the seeded generator in help_gb300):
  ref_kernels.npz   CSRMV_N / CSRMV_T (Helper.cpp:57-81), RenewPartialCholesky
                    (PCG.cpp:38-177) and Preconditioner (PCG.cpp:183-196) outputs,
                    ADAt_Allocate + ADAt_Calc (Helper.cpp:215-348) output, and one
                    SolveLinearEquation (UsePCG_CPU.cpp:91-183) with its CG count.
  ref_hsd_small.npz every SolveLinearEquation call (d, b_1, b_2, x_1, x_2, CG
                    iterations) of the reference program solving a 50 x 150 LP.
  ref_hsd.json      the reference program's iteration table (P.Obj, D.Obj, gap,
                    infeasibilities as printed) for three LPs incl. config 0,
                    and its final iterate at full precision (status, iterations,
                    objectives, gap, infeasibilities, tau, kappa; written by
                    oracle/ref/ref_record.cpp when HSD_Main destructs the
                    backend, HSDSolver.cpp:881).
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from help_gb300 import lp as L  # noqa: E402
from oracle import bindings as ob  # noqa: E402

P = ob.P


def kernels():
    R = ob.ref()
    lp = L.generate(L.spec_random(40, 120, 5), 11)
    m, n = lp.m, lp.n
    rng = np.random.default_rng(5)
    R.ref_load(m, n, P(lp.col_ptr), P(lp.row_ind), P(lp.val))
    R.ref_construct()
    rp, ci, v = lp.csr()
    x_n = rng.standard_normal(n)
    x_t = rng.standard_normal(m)
    y0 = rng.standard_normal(m)
    yN = y0.copy()
    beg, end = rp[:-1].copy(), rp[1:].copy()
    R.ref_csrmv_n(m, n, 1.5, P(v), P(ci), P(beg), P(end), P(x_n), -0.5, P(yN))
    yT = np.zeros(n)
    R.ref_csrmv_t(m, n, 1.0, P(v), P(ci), P(beg), P(end), P(x_t), 0.0, P(yT))
    d = np.exp(rng.uniform(-4, 4, n))
    kk = R.ref_pchol_cols()
    perm = np.zeros(m, np.int32)
    Lm = np.zeros(m * kk)
    D = np.zeros(kk)
    ds = np.zeros(m)
    R.ref_pchol(P(d), 0.0, 0.0, P(perm), P(Lm), P(D), P(ds))
    r_perm = rng.standard_normal(m)
    z_perm = np.zeros(m)
    R.ref_precond(P(r_perm), P(z_perm))
    cap = 100000
    arp = np.zeros(m + 1, np.int32)
    acol = np.zeros(cap, np.int32)
    aval = np.zeros(cap)
    w = np.exp(rng.uniform(-2, 2, n))
    nz = R.ref_adat(P(w), P(arp), P(acol), P(aval), cap)
    b1 = rng.standard_normal(n)
    b2 = rng.standard_normal(m)
    x1 = np.zeros(n)
    x2 = np.zeros(m)
    it = R.ref_solve(P(d), P(b1), P(b2), P(x1), P(x2))
    np.savez_compressed(
        os.path.join(HERE, "ref_kernels.npz"), gen=np.array([40, 120, 5, 11]), x_n=x_n, x_t=x_t, y0=y0,
        yN=yN, yT=yT, d=d, k=np.array(kk), perm=perm, L=Lm.reshape(m, kk), D=D, diag_s=ds, r_perm=r_perm,
        z_perm=z_perm, w=w, adat_rp=arp, adat_col=acol[:nz], adat_val=aval[:nz], b1=b1, b2=b2, x1=x1, x2=x2,
        iters=np.array(it))


def read_solves(path):
    out = {"d": [], "b1": [], "b2": [], "x1": [], "x2": [], "iters": []}
    with open(path, "rb") as f:
        while True:
            hdr = f.read(8)
            if len(hdr) < 8:
                break
            m, n = np.frombuffer(hdr, np.int32)
            it = np.frombuffer(f.read(8), np.int64)[0]
            for key, cnt in (("d", n), ("b1", n), ("b2", m), ("x1", n), ("x2", m)):
                out[key].append(np.frombuffer(f.read(8 * cnt), np.float64).copy())
            out["iters"].append(it)
    return {k: np.array(v) for k, v in out.items()}


ROW = re.compile(r"^\|\s*(\d+)\s*\|\s*(\S+)\s*\|\s*(\S+)\s*\|\s*(\S+)\s*\|\s*(\S+)\s*\|\s*(\S+)\s*\|")


def run_ref_program(lp, record: bool):
    with tempfile.TemporaryDirectory() as tmp:
        mps = os.path.join(tmp, "lp.mps")
        lp.write_mps(mps)
        env = dict(os.environ)
        if record:
            env["HELP_REF_RECORD"] = tmp
        env["HELP_REF_FINAL"] = os.path.join(tmp, "final.txt")
        r = subprocess.run([ob.REF_BIN, mps], input="x\n", capture_output=True, text=True, cwd=tmp, env=env,
                           timeout=3600)
        rows = []
        for line in r.stdout.splitlines():
            mm = ROW.match(line)
            if mm:
                rows.append([int(mm.group(1))] + [float(mm.group(i)) for i in range(2, 7)])
        solves = read_solves(os.path.join(tmp, "solves.bin")) if record else None
        status = [l for l in r.stdout.splitlines() if "Problem Status" in l]
        final = {}
        with open(env["HELP_REF_FINAL"]) as f:
            for line in f:
                key, val = line.split()
                final[key] = int(val) if key in ("status", "iterations", "solves", "cg_iterations") else float(val)
        return rows, solves, (status[0] if status else ""), final


def hsd():
    tables = {}
    cases = [("random-50x150-k5-seed1", L.spec_random(50, 150, 5), 1),
             ("random-200x600-k5-seed2", L.spec_random(200, 600, 5), 2),
             ("config0-seed0", L.CONFIGS[0][0](), 0)]
    for name, spec, seed in cases:
        lp = L.generate(spec, seed)
        record = name.startswith("random-50x150")
        rows, solves, status, final = run_ref_program(lp, record)
        tables[name] = {"m": lp.m, "n": lp.n, "seed": seed, "rows": rows, "status": status,
                        "cg_iters": solves["iters"].tolist() if solves is not None else None,
                        "final": final}
        if solves is not None:
            np.savez_compressed(os.path.join(HERE, "ref_hsd_small.npz"), **solves)
        print(name, len(rows), "rows", status)
    with open(os.path.join(HERE, "ref_hsd.json"), "w") as f:
        json.dump(tables, f, indent=1)


if __name__ == "__main__":
    if not ob.ref_available():
        sys.exit("reference harness not built (make -C oracle/ref)")
    kernels()
    hsd()
