"""The learned part: per-row MLP giving a Schur-diagonal correction and a
warm-start scale for the normal-equations PCG (include/help_gpu.h, HELP_MLP_*).

Pipeline, all on the GPU through the library's own kernels:
  1. ``collect``: run the HSD interior-point method with the plain FP64 PCG
     backend on seeded LPs; after every renew record the raw per-row features
     of every solve slot (device kernel, help_pcg_features), the pivots and
     the solutions x_2 of every solve slot;
  2. ``targets``: per row, (0) the log-ratio of a 2-norm equilibrated diagonal
     of the Schur complement S (non-pivot block) to diag(S) -- computed from
     the dense S, so for small systems only -- and (1) the per-row scale s of
     the previous renew's x_2 of the same slot that minimises the G-norm
     error to this renew's x_2 (ridge toward the best single scalar; dense G,
     again small systems only);
  3. ``train``: full-batch Adam on the weighted squared error with the
     library's BF16 forward / backward kernels (help_mlp_train_step);
  4. ``evaluate``: the same IPM with and without the model attached.

Instances are scaled-down multicommodity-flow LPs of the benchmark's family
(grid graphs, several commodities); the dense targets bound their size.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import native
from .backend import GpuNormalEquations, GpuPairNormalEquations


FEATURES = 11   # features in use per row (include/help_gpu.h); the rest of the 16 are zero
SLOTS = 4       # solve slots after a renew that get their own features


def _torch():
    import torch

    return torch


def bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> BF16 bit patterns (uint16), round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


class Mlp:
    """A model on one GPU (help_mlp)."""

    def __init__(self, device: int = 0, params: np.ndarray | None = None):
        self.lib = native.gpu_lib()
        h = C.c_void_p()
        rc = self.lib.help_mlp_create(device, C.byref(h))
        if rc != native.HELP_OK:
            raise RuntimeError("help_mlp_create failed (%d)" % rc)
        self.h = h
        self.device = device
        if params is not None:
            self.set_params(params)

    def _check(self, rc: int) -> None:
        if rc != native.HELP_OK:
            raise RuntimeError("help_mlp: %s (%d)" % (self.lib.help_mlp_last_error(self.h).decode(), rc))

    def close(self) -> None:
        if self.h:
            self.lib.help_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (native.MLP_PARAMS,)
        self._check(self.lib.help_mlp_set_params(self.h, p.ctypes.data))

    def get_params(self) -> np.ndarray:
        p = np.empty(native.MLP_PARAMS, np.float32)
        self._check(self.lib.help_mlp_get_params(self.h, p.ctypes.data))
        return p

    # device tensors (torch) in, as the C ABI takes device pointers
    def forward(self, x_bits, rows: int):
        torch = _torch()
        out = torch.empty((rows, native.MLP_OUT), dtype=torch.float32, device=x_bits.device)
        self._check(self.lib.help_mlp_forward(self.h, x_bits.data_ptr(), rows, out.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        return out

    def loss_grad(self, x_bits, t, w, rows: int):
        loss = C.c_double()
        g = np.empty(native.MLP_OFF_MEAN, np.float32)
        self._check(self.lib.help_mlp_loss_grad(self.h, x_bits.data_ptr(), t.data_ptr(), w.data_ptr(), rows,
                                                C.byref(loss), g.ctypes.data))
        return loss.value, g

    def train_step(self, x_bits, t, w, rows: int, lr: float) -> float:
        loss = C.c_double()
        self._check(self.lib.help_mlp_train_step(self.h, x_bits.data_ptr(), t.data_ptr(), w.data_ptr(), rows,
                                                 C.c_float(lr), C.byref(loss)))
        return loss.value


def init_params(seed: int, mean=None, scale=None) -> np.ndarray:
    """He-style initial weights, zero biases except the warm-start scale's (1)."""
    rng = np.random.default_rng(seed)
    In, H, O = native.MLP_IN, native.MLP_HIDDEN, native.MLP_OUT
    p = np.zeros(native.MLP_PARAMS, np.float32)
    p[native.MLP_OFF_W1:native.MLP_OFF_B1] = rng.normal(0, np.sqrt(2.0 / In), H * In)
    p[native.MLP_OFF_W2:native.MLP_OFF_B2] = rng.normal(0, np.sqrt(2.0 / H), H * H)
    p[native.MLP_OFF_W3:native.MLP_OFF_B3] = rng.normal(0, 0.1 * np.sqrt(1.0 / H), O * H)
    p[native.MLP_OFF_B3 + 1] = 1.0
    p[native.MLP_OFF_MEAN:native.MLP_OFF_SCALE] = 0.0 if mean is None else mean
    p[native.MLP_OFF_SCALE:] = 1.0 if scale is None else scale
    return p


def fixed_warm_params() -> np.ndarray:
    """No network: no diagonal correction, warm-start scale 1 (the previous
    renew's solution of the same slot, re-fitted by the optimal scalar)."""
    p = zero_params()
    p[native.MLP_OFF_B3 + 1] = 1.0
    return p


def diag_head_only(params: np.ndarray) -> np.ndarray:
    """The trained network's Schur-diagonal correction with the warm-start
    head replaced by the constant 1 (the warm start without the network)."""
    p = np.array(params, np.float32, copy=True)
    p[native.MLP_OFF_W3 + native.MLP_HIDDEN:native.MLP_OFF_W3 + 2 * native.MLP_HIDDEN] = 0.0  # W3 is [out][hidden]
    p[native.MLP_OFF_B3 + 1] = 1.0
    return p


def warm_head_only(params: np.ndarray) -> np.ndarray:
    """The trained network's warm-start scales with no diagonal correction."""
    p = np.array(params, np.float32, copy=True)
    p[native.MLP_OFF_W3:native.MLP_OFF_W3 + native.MLP_HIDDEN] = 0.0
    p[native.MLP_OFF_B3] = 0.0
    return p


def zero_params() -> np.ndarray:
    """A model whose outputs are 0: no correction, no warm start (alpha = 0)."""
    p = np.zeros(native.MLP_PARAMS, np.float32)
    p[native.MLP_OFF_SCALE:] = 1.0
    return p


class _Recorder:
    """NeBackend whose entry points call a GPU backend and record each renew."""

    def __init__(self, ne: GpuNormalEquations, m: int, n: int):
        self.ne, self.m, self.n = ne, m, n
        self.renews: list[dict] = []
        torch = _torch()
        self._feat = torch.empty((m, native.MLP_IN), dtype=torch.float32, device="cuda:%d" % ne.options.device)
        lib, ctx = ne.lib, ne.ctx
        self.error: BaseException | None = None

        def guarded(fn):
            # an exception must not cross the C driver: keep it, report failure
            def call(*a):
                try:
                    return fn(*a)
                except BaseException as e:  # noqa: BLE001
                    self.error = e
                    return native.HELP_E_ARG
            return call

        @guarded
        def construct(_c, m_, n_, cp, ri, v):
            ne.m, ne.n = int(m_), int(n_)
            return lib.help_pcg_construct(ctx, m_, n_, cp, ri, v)

        @guarded
        def renew(_c, d):
            rc = lib.help_pcg_renew(ctx, d)
            if rc == native.HELP_OK:
                self._snapshot(d)
            return rc

        @guarded
        def solve(_c, d, b1, b2, x1, x2):
            rc = lib.help_pcg_solve(ctx, d, b1, b2, x1, x2)
            if rc == native.HELP_OK and self.renews:
                x = np.ctypeslib.as_array(C.cast(x2, C.POINTER(C.c_double)), (self.m,)).copy()
                self.renews[-1]["x2"].append(x)
            return rc

        @guarded
        def destruct(_c):
            return lib.help_pcg_destruct(ctx)

        @guarded
        def matvec(_c, t, s, v, dest):
            return lib.help_pcg_matvec_acc(ctx, t, s, v, dest)

        self._fns = (native.CONSTRUCT_FN(construct), native.RENEW_FN(renew), native.SOLVE_FN(solve),
                     native.DESTRUCT_FN(destruct), native.MATVEC_FN(matvec))

    def _snapshot(self, d_ptr) -> None:
        ne = self.ne
        feats = []
        for slot in range(SLOTS):
            rc = ne.lib.help_pcg_features(ne.ctx, slot, self._feat.data_ptr())
            if rc != native.HELP_OK:
                raise RuntimeError("help_pcg_features failed (%d)" % rc)
            feats.append(self._feat.cpu().numpy().copy())
        piv, dg, ds = ne.pivots()
        d = np.ctypeslib.as_array(C.cast(d_ptr, C.POINTER(C.c_double)), (self.n,)).copy()
        self.renews.append({"feat": feats, "piv": piv.copy(), "diag": dg.copy(), "ds": ds.copy(), "d": d, "x2": []})

    def backend(self) -> native.NeBackend:
        f = lambda fn: C.cast(fn, C.c_void_p).value
        return native.NeBackend(ctx=None, construct=f(self._fns[0]), renew=f(self._fns[1]), solve=f(self._fns[2]),
                                destruct=f(self._fns[3]), matvec=f(self._fns[4]))


def collect(lp, pivots: int, cg_tol: float = 1e-10, device: int = 0, max_seconds: float = 0.0,
            cg_max_iter: int = 200_000, cap_ok: bool = False) -> list[dict]:
    """Renews of one IPM run of ``lp`` with the plain PCG (a zero model attached
    so the solutions of every slot are kept for the next renew's features);
    ``max_seconds`` > 0 keeps the renews reached within that time."""
    from . import hsd

    zero = Mlp(device, zero_params())
    with GpuNormalEquations(pivots=pivots, cg_tol=cg_tol, cg_max_iter=cg_max_iter, device=device,
                            cap_ok=cap_ok) as ne:
        ne._check(ne.lib.help_pcg_attach_mlp(ne.ctx, zero.h))
        rec = _Recorder(ne, lp.m, lp.n)
        res = hsd.solve_lp(lp, rec.backend(), max_seconds=max_seconds)
        ne._check(ne.lib.help_pcg_attach_mlp(ne.ctx, None))
    zero.close()
    if rec.error is not None:
        raise RuntimeError("recording the IPM run failed: %r" % (rec.error,)) from rec.error
    if res["rc"] != 0 or res["status"] not in ((0, 2) if max_seconds > 0 else (0,)):
        raise RuntimeError("IPM failed while collecting (rc %d, status %d)" % (res["rc"], res["status"]))
    return rec.renews


def _dense(lp) -> np.ndarray:
    A = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        A[lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]], j] = lp.val[lp.col_ptr[j]:lp.col_ptr[j + 1]]
    return A


def equilibrated_log_ratio(S: np.ndarray, iters: int = 8) -> np.ndarray:
    """ln(e_i / S_ii) for the diagonal e that 2-norm-equilibrates S symmetrically."""
    e = np.diag(S).copy()
    for _ in range(iters):
        sc = 1.0 / np.sqrt(e)
        rn = np.sqrt(((S * sc[None, :] * sc[:, None]) ** 2).sum(1))
        e = e * rn
    return np.log(e / np.diag(S))


def energy_scale_target(G: np.ndarray, xp: np.ndarray, xc: np.ndarray, ridge: float = 100.0) -> np.ndarray:
    """Per-row scale s of the warm start s .* xp that minimises the G-norm
    error || s .* xp - xc ||_G (the quantity CG's convergence follows), with
    a ridge pulling s toward the best single scalar a*; returned as s / a*,
    since the solver re-fits the scalar itself.  The ridge is relative to the
    mean diagonal of diag(xp) G diag(xp); on held-out multicommodity-flow LPs
    ridge 0.1 gave per-row targets (std 0.77) the features cannot predict,
    and the warm start lost to a plain scale of 1; 100 keeps the targets
    within ~0.07 of 1."""
    gx = G @ xp
    den = float(xp @ gx)
    if not den > 0:
        return np.ones_like(xp)
    a = float(xc @ gx) / den
    M = (xp[:, None] * G) * xp[None, :]
    lam = ridge * max(np.trace(M) / len(xp), 1e-300)
    s = np.linalg.solve(M + lam * np.eye(len(xp)), xp * (G @ xc) + lam * a)
    return s / a if a != 0 else np.ones_like(xp)


def targets(lp, renews: list[dict], dense_max: int = 4000, diag: bool = True) -> dict:
    """Training rows (raw features, targets, weights) of one IPM run.  Output
    0: the equilibration log-ratio of the Schur diagonal (weight 0 with
    ``diag=False``); output 1: the G-norm-optimal warm-start scale."""
    if lp.m > dense_max:
        raise ValueError("dense Schur targets need m <= %d" % dense_max)
    A = _dense(lp)
    X, T, W = [], [], []
    for r in range(1, len(renews)):
        cur, prev = renews[r], renews[r - 1]
        G = (A / cur["d"]) @ A.T
        piv = cur["piv"]
        mask = np.ones(lp.m, bool)
        mask[piv] = False
        N = np.where(mask)[0]
        t0 = np.zeros(lp.m)
        if diag:
            if len(piv):
                Wi = np.linalg.inv(G[np.ix_(piv, piv)])
                Cn = G[np.ix_(N, piv)]
                S = G[np.ix_(N, N)] - Cn @ Wi @ Cn.T
            else:
                S = G[np.ix_(N, N)]
            t0[N] = equilibrated_log_ratio(S)
        for s in range(min(len(cur["x2"]), len(prev["x2"]))):
            xp, xc = prev["x2"][s], cur["x2"][s]
            if not (xp @ xp) > 0:
                continue
            t1 = np.clip(energy_scale_target(G, xp, xc), -4.0, 4.0)
            t = np.stack([t0, t1], 1)
            w0 = mask / max(len(N), 1) if (s == 0 and diag) else np.zeros(lp.m)
            w = np.stack([w0, np.full(lp.m, 1.0 / lp.m)], 1)
            X.append(cur["feat"][min(s, SLOTS - 1)])
            T.append(t)
            W.append(w)
    return {"X": np.concatenate(X).astype(np.float32), "T": np.concatenate(T).astype(np.float32),
            "W": np.concatenate(W).astype(np.float32)}


def energy_scale_target_sparse(A, d: np.ndarray, xp: np.ndarray, xc: np.ndarray, ridge: float = 100.0,
                               tol: float = 1e-8, maxiter: int = 2000) -> np.ndarray:
    """energy_scale_target with G = A D^-1 A^T applied as two sparse products
    (A: scipy CSR), for systems too large for a dense G: the ridge system
    (diag(xp) G diag(xp) + lam I) s = diag(xp) G xc + lam a* solved by
    Jacobi-preconditioned CG (its diagonal: xp^2 diag(G) + lam)."""
    from scipy.sparse.linalg import LinearOperator, cg

    dinv = 1.0 / d
    G = lambda v: A @ (dinv * (A.T @ v))
    gx = G(xp)
    den = float(xp @ gx)
    if not den > 0:
        return np.ones_like(xp)
    a = float(xc @ gx) / den
    dg = np.asarray(A.multiply(A) @ dinv).ravel()
    diagM = xp * xp * dg
    lam = ridge * max(float(diagM.mean()), 1e-300)
    op = LinearOperator((len(xp), len(xp)), matvec=lambda v: xp * G(xp * v) + lam * v, dtype=np.float64)
    pre = LinearOperator((len(xp), len(xp)), matvec=lambda v: v / (diagM + lam), dtype=np.float64)
    s, _ = cg(op, xp * G(xc) + lam * a, x0=np.full(len(xp), a), rtol=tol, maxiter=maxiter, M=pre)
    return s / a if a != 0 else np.ones_like(xp)


def targets_sparse(lp, renews: list[dict], ridge: float = 100.0) -> dict:
    """Training rows of one IPM run with the warm-start head only (output 1,
    the G-norm-optimal per-row scale, from sparse products); output 0 (the
    Schur-diagonal head, which needs the dense Schur complement) is given
    weight 0.  For flows of any size."""
    from scipy.sparse import csr_matrix

    rp, ci, v = lp.csr()
    A = csr_matrix((v, ci, rp), shape=(lp.m, lp.n))
    X, T, W = [], [], []
    for r in range(1, len(renews)):
        cur, prev = renews[r], renews[r - 1]
        for s in range(min(len(cur["x2"]), len(prev["x2"]))):
            xp, xc = prev["x2"][s], cur["x2"][s]
            if not (xp @ xp) > 0:
                continue
            t1 = np.clip(energy_scale_target_sparse(A, cur["d"], xp, xc, ridge), -4.0, 4.0)
            X.append(cur["feat"][min(s, SLOTS - 1)])
            T.append(np.stack([np.zeros(lp.m), t1], 1))
            W.append(np.stack([np.zeros(lp.m), np.full(lp.m, 1.0 / lp.m)], 1))
    return {"X": np.concatenate(X).astype(np.float32), "T": np.concatenate(T).astype(np.float32),
            "W": np.concatenate(W).astype(np.float32)}


def normalisation(X: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    mean = np.zeros(native.MLP_IN, np.float32)
    scale = np.ones(native.MLP_IN, np.float32)
    mean[:FEATURES] = X[:, :FEATURES].mean(0)
    sd = X[:, :FEATURES].std(0)
    scale[:FEATURES] = np.where(sd > 1e-6, 1.0 / np.maximum(sd, 1e-6), 1.0)
    return mean, scale


def normalise_bits(X: np.ndarray, mean: np.ndarray, scale: np.ndarray) -> np.ndarray:
    """The device feature kernel's normalisation and BF16 rounding, on the host."""
    Z = ((X.astype(np.float32) - mean) * scale).astype(np.float32)
    Z[:, FEATURES:] = 0.0
    return bf16_bits(Z)


def train(data: dict, steps: int = 600, lr: float = 3e-3, seed: int = 0, device: int = 0,
          log=None) -> tuple[np.ndarray, list[float]]:
    """Full-batch Adam with the library's kernels; returns (params, losses)."""
    torch = _torch()
    mean, scale = normalisation(data["X"])
    p0 = init_params(seed, mean, scale)
    mlp = Mlp(device, p0)
    dev = torch.device("cuda", device)
    xb = torch.from_numpy(normalise_bits(data["X"], mean, scale).view(np.int16)).to(dev)
    t = torch.from_numpy(data["T"]).to(dev)
    w = torch.from_numpy(data["W"]).to(dev)
    rows = data["X"].shape[0]
    losses = []
    for it in range(steps):
        step_lr = lr * (0.1 ** (it / max(steps, 1)))
        losses.append(mlp.train_step(xb, t, w, rows, step_lr))
        if log and (it % 100 == 0 or it == steps - 1):
            log("step %d loss %.6g" % (it, losses[-1]))
    params = mlp.get_params()
    mlp.close()
    return params, losses


def evaluate(lp, pivots: int, params: np.ndarray | None, cg_tol: float = 1e-10, device: int = 0,
             precision: str = "fp64", max_seconds: float = 0.0, cg_max_iter: int = 200_000,
             cap_ok: bool = False, trace: bool = False, paired: bool = False) -> dict:
    """One IPM run; with ``params`` the model is attached; precision "mixed"
    runs the FP32-in-FP64-refinement form (refined to cg_tol).
    ``max_seconds`` caps the run's wall time; ``cap_ok`` lets a solve that
    stops at ``cg_max_iter`` hand back its inexact direction; ``trace``
    records (seconds, rel gap, primal / dual infeasibility, CG iterations so
    far) at every iteration.  ``paired``: the bottom system and the first
    direction of every iteration solved together on two contexts
    (GpuPairNormalEquations), the model attached to both: the pair maps
    each system to the solve slot it takes on one context and hands context
    1 the bottom system's solution before each renew, so the run is the
    single context's."""
    from . import hsd

    mlp = Mlp(device, params) if params is not None else None
    rows = []
    kw = dict(pivots=pivots, cg_tol=cg_tol, cg_max_iter=cg_max_iter, device=device, precision=precision,
              ir_tol=cg_tol, cap_ok=cap_ok)
    with (GpuPairNormalEquations(**kw) if paired else GpuNormalEquations(**kw)) as ne:
        lib = ne.lib
        ctxs = [ne.context(0), ne.context(1)] if paired else [ne.ctx]
        stats = (lambda: [ne.stats(0), ne.stats(1)]) if paired else (lambda: [ne.stats()])
        total = lambda key: int(sum(s_[key] for s_ in stats()))

        def attach(h):
            for c in ctxs:
                rc = lib.help_pcg_attach_mlp(c, h)
                if rc != native.HELP_OK:
                    raise RuntimeError("help_pcg_attach_mlp failed (%d)" % rc)

        if mlp is not None:
            attach(mlp.h)
        t0 = time.perf_counter()

        def on_iter(it, s):
            rows.append([round(time.perf_counter() - t0, 3), s[2], s[3], s[4], total("cg_iterations_total")])

        r = hsd.solve_lp(lp, ne.ne_backend(), max_seconds=max_seconds, on_iter=on_iter if trace else None)
        wall = time.perf_counter() - t0
        cg_total, fallbacks = total("cg_iterations_total"), total("learned_fallbacks")
        if mlp is not None:
            attach(None)
    if mlp is not None:
        mlp.close()
    if r["rc"] != 0:
        raise RuntimeError("IPM backend error (rc %d)" % r["rc"])
    out = {"status": r["status"], "iterations": r["iterations"], "primal_obj": r["primal_obj"],
           "rel_gap": r["rel_gap"], "primal_infeas": r["primal_infeas"], "dual_infeas": r["dual_infeas"],
           "cg_iterations": cg_total, "seconds": wall, "learned_fallbacks": fallbacks}
    if trace:
        out["trace"] = {"columns": ["s", "rel_gap", "primal_infeas", "dual_infeas", "cg_iterations"], "rows": rows}
    return out


def scaling_study(grid: int, commodities: int, pairs: int, train_seeds, held_out, pivots: int = 16,
                  steps: int = 400, device: int = 0, full_size: dict | None = None) -> dict:
    """The warm-start head trained on the IPM iterates of flows far past the
    dense-Schur limit (targets from sparse products, targets_sparse), and its
    effect on held-out seeds: whole-IPM CG iterations and seconds of the
    plain PCG, of the same warm start without the network (fixed_warm_params)
    and of the trained network (warm head only).  ``full_size`` (keys grid,
    commodities, pairs, seed, pivots, seconds) adds the benchmark's full flow
    run under a wall-clock cap, compared at the last interior-point
    iteration every arm reached."""
    from . import lp as L

    spec = dict(grid=grid, commodities=commodities, pairs=pairs)
    t0 = time.perf_counter()
    data = []
    for s in train_seeds:
        lp = L.generate(L.spec_mcf(**spec), s)
        data.append(targets_sparse(lp, collect(lp, pivots, device=device)))
    train_set = {k: np.concatenate([d[k] for d in data]) for k in ("X", "T", "W")}
    collect_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    params, losses = train(train_set, steps=steps, device=device)
    params = warm_head_only(params)
    out = {"flow": "%d x %d grid, %d commodities" % (grid, grid, commodities), "pivots": pivots,
           "train_seeds": list(train_seeds), "train_rows": int(train_set["X"].shape[0]),
           "collect_s": round(collect_s, 1), "train_s": round(time.perf_counter() - t0, 2),
           "loss_first": losses[0], "loss_last": losses[-1], "held_out": []}
    arms = (("plain", None), ("fixed_warm_start", fixed_warm_params()), ("learned", params))
    for s in held_out:
        lp = L.generate(L.spec_mcf(**spec), s)
        row = {"seed": s, "m": lp.m, "n": lp.n}
        for name, prm in arms:
            r = evaluate(lp, pivots, prm, device=device)
            row[name] = {"cg": r["cg_iterations"], "s": round(r["seconds"], 3), "status": r["status"],
                         "iterations": r["iterations"], "primal_obj": r["primal_obj"]}
        out["held_out"].append(row)
    if full_size:
        fs = dict(full_size)
        lp = L.generate(L.spec_mcf(fs["grid"], fs["commodities"], fs["pairs"]), fs["seed"])
        runs = {name: evaluate(lp, fs["pivots"], prm, device=device, max_seconds=fs["seconds"], cg_tol=1e-8,
                               cg_max_iter=50_000, cap_ok=True, trace=True) for name, prm in arms}
        last = min(len(r["trace"]["rows"]) for r in runs.values())
        out["full_size"] = {"flow": "%d x %d grid, %d commodities, seed %d (m=%d, n=%d)" % (
            fs["grid"], fs["grid"], fs["commodities"], fs["seed"], lp.m, lp.n), "pivots": fs["pivots"],
            "cap_s": fs["seconds"], "compared_at_iteration": last - 1}
        for name, r in runs.items():
            row = r["trace"]["rows"][last - 1]
            out["full_size"][name] = {"s": row[0], "rel_gap": row[1], "cg": row[4],
                                      "iterations_reached": r["iterations"], "final_rel_gap": r["rel_gap"]}
    return out
