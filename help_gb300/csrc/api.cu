// C ABI of libhelp_gpu.so (declared in include/help_gpu.h).
//
// Boundary: the reference's PCG backend (UsePCG_CPU.cpp:26-183 + PCG.cpp).
// Host arrays in, host arrays out; everything else stays on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "context.h"
#include "guard.h"
#include "mlp.h"
#include "items.h"
#include "kernels.h"
#include "spmv.cuh"

using namespace help;

// model internals for the solver (mlp_api.cu)
const help::MlpDevWeights* help_mlp_device_weights(const help_mlp* mlp);
int help_mlp_device(const help_mlp* mlp);

namespace {

constexpr int kPartElems = 8192;  // per-block partial sums and reduction scratch

int fail(help_pcg* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}
int fail_cuda(help_pcg* ctx, cudaError_t e, const char* what) {
    if (ctx) ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? HELP_E_NOMEM : HELP_E_CUDA;
}

#define CK(call)                                                  \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return fail_cuda(ctx, _e, #call); \
    } while (0)

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

DevCtrl* ctrl_of(help_pcg* ctx) { return ctx->ctrl.as<DevCtrl>(); }

int upload_split(help_pcg* ctx, RowSplit& S, const int32_t* ptr, int32_t rows, int g_min, int per_lane,
                 const int32_t* idx, size_t elem, double order_waste) {
    RowPlanHost h = plan_rows(ptr, rows, g_min, per_lane, order_waste);
    S.n_sell = 0;
    if (idx) {
        SellHost sh = plan_sell(ptr, idx, rows, h.short_max);
        if (sh.nslices > 0) {
            const size_t ne = sh.idx.size();
            CK(S.sell_ptr.ensure(4 * sh.ptr.size()));
            CK(S.sell_perm.ensure(4 * sh.perm.size()));
            CK(S.sell_idx.ensure(4 * ne));
            CK(S.sell_map.ensure(4 * ne));
            CK(S.sell_val.ensure(elem * ne));
            CK(cudaMemcpyAsync(S.sell_ptr.p, sh.ptr.data(), 4 * sh.ptr.size(), cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaMemcpyAsync(S.sell_perm.p, sh.perm.data(), 4 * sh.perm.size(), cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaMemcpyAsync(S.sell_idx.p, sh.idx.data(), 4 * ne, cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaMemcpyAsync(S.sell_map.p, sh.map.data(), 4 * ne, cudaMemcpyHostToDevice, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));  // sh goes out of scope
            S.n_sell = sh.nslices;
            S.sell_W = sh.W;
            S.sell_entries = (int64_t)ne;
        }
    }
    S.G = h.G;
    S.short_max = h.short_max;
    S.n_med = (int32_t)h.med.size();
    S.n_long = (int32_t)h.lng.size();
    S.n_seg = (int32_t)(h.seg.size() / 4);
    S.n_short = (int32_t)h.short_order.size();
    if (S.n_short > 0) {
        CK(S.sorder.ensure(4 * (size_t)S.n_short));
        CK(cudaMemcpyAsync(S.sorder.p, h.short_order.data(), 4 * (size_t)S.n_short, cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    CK(S.med.ensure(4 * std::max<size_t>(h.med.size(), 1)));
    CK(S.lng.ensure(4 * std::max<size_t>(h.lng.size(), 1)));
    CK(S.seg.ensure(4 * std::max<size_t>(h.seg.size(), 4)));
    CK(S.lnseg.ensure(4 * std::max<size_t>(h.lng.size(), 1)));
    CK(S.lbase.ensure(4 * std::max<size_t>(h.lng.size(), 1)));
    CK(S.tickets.ensure(4 * std::max<size_t>(h.lng.size(), 1)));
    CK(S.parts.ensure(8 * std::max<size_t>((size_t)h.n_parts, 1)));
    if (!h.med.empty()) CK(cudaMemcpyAsync(S.med.p, h.med.data(), 4 * h.med.size(), cudaMemcpyHostToDevice, ctx->stream));
    if (!h.lng.empty()) {
        CK(cudaMemcpyAsync(S.lng.p, h.lng.data(), 4 * h.lng.size(), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(S.seg.p, h.seg.data(), 4 * h.seg.size(), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(S.lnseg.p, h.long_nseg.data(), 4 * h.lng.size(), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(S.lbase.p, h.long_base.data(), 4 * h.lng.size(), cudaMemcpyHostToDevice, ctx->stream));
        // the last CTA of a row resets its ticket, so zero once here
        CK(cudaMemsetAsync(S.tickets.p, 0, 4 * h.lng.size(), ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));  // h goes out of scope
    return HELP_OK;
}

// idx (host column indices, may be null): also lay the short rows out in
// slices for B's products (A and A^T, whose B values are refreshed at renew)
int upload_plan(help_pcg* ctx, RowPlan& P, const int32_t* ptr, int32_t rows, bool with_f32,
                const int32_t* idx = nullptr, int per_lane64 = kPerLaneF64, int per_lane32 = kPerLaneF32,
                double order_waste = kOrderWaste) {
    P.rows = rows;
    int rc = upload_split(ctx, P.s64, ptr, rows, kGminF64, per_lane64, idx, 8, order_waste);
    if (!rc && with_f32) rc = upload_split(ctx, P.s32, ptr, rows, kGminF32, per_lane32, idx, 4, order_waste);
    return rc;
}

// B's values into the sliced layouts of A and A^T (both precisions present)
int refresh_sell(help_pcg* ctx, bool mixed) {
    const struct {
        RowSplit* S;
        const DevMem* src;
        bool f32;
    } jobs[4] = {{&ctx->pl_csr.s64, &ctx->bv, false},
                 {&ctx->pl_csc.s64, &ctx->bvT, false},
                 {&ctx->pl_csr.s32, &ctx->bv32, true},
                 {&ctx->pl_csc.s32, &ctx->bvT32, true}};
    for (const auto& j : jobs) {
        if (j.f32 && !mixed) continue;
        if (j.S->n_sell <= 0) continue;
        if (j.f32)
            CK(sell_gather<float>(j.S->sell_map.as<int>(), j.src->as<float>(), j.S->sell_val.as<float>(),
                                  j.S->sell_entries, ctx->num_sms, ctx->stream));
        else
            CK(sell_gather<double>(j.S->sell_map.as<int>(), j.src->as<double>(), j.S->sell_val.as<double>(),
                                   j.S->sell_entries, ctx->num_sms, ctx->stream));
    }
    return HELP_OK;
}

// sell: the value array is B's (bv / bvT / their FP32 copies), whose sliced
// copy the split holds; other value arrays (A's own) take the CSR rows
template <class V>
SpmvView<V> view(const RowPlan& P, const DevMem& ptr, const DevMem& idx, const DevMem& val, bool sell = false) {
    const RowSplit& S = std::is_same<V, float>::value ? P.s32 : P.s64;
    SpmvView<V> v;
    v.rows = P.rows;
    v.G = S.G;
    v.short_max = S.short_max;
    v.n_med = S.n_med;
    v.n_long = S.n_long;
    v.ptr = ptr.as<int>();
    v.idx = idx.as<int>();
    v.val = val.as<V>();
    v.med_rows = S.med.as<int>();
    v.long_rows = S.lng.as<int>();
    v.n_seg = S.n_seg;
    v.segs = S.seg.as<int4>();
    v.long_nseg = S.lnseg.as<int>();
    v.long_base = S.lbase.as<int>();
    v.tickets = S.tickets.as<unsigned int>();
    v.parts = S.parts.as<double>();
    v.short_order = S.n_short > 0 ? S.sorder.as<int>() : nullptr;
    v.n_short = S.n_short;
    if (sell && S.n_sell > 0) {
        v.n_sell = S.n_sell;
        v.sell_W = S.sell_W;
        v.sell_ptr = S.sell_ptr.as<int>();
        v.sell_perm = S.sell_perm.as<int>();
        v.sell_idx = S.sell_idx.as<int>();
        v.sell_val = S.sell_val.as<V>();
    }
    return v;
}

// Standalone passes (grid-stride).  At scale, one wave of resident CTAs: a
// grid past the resident count leaves a partial second wave (config 4's
// product, 104M nonzeros: 3,094 -> 3,440 GB/s with one wave; the HSD
// driver's A v 0.98 -> 0.87 ms).  Small passes keep 8 CTAs per SM, whose
// extra blocks even out the few slices each block takes (config 1, 3.2M
// nonzeros: 2,018 GB/s against 1,937 with one wave).
constexpr int64_t kOneWaveNnz = 32 << 20;
int spmv_blocks(help_pcg* ctx) {
    return ctx->num_sms * (ctx->nnz >= kOneWaveNnz ? spmv_blocks_per_sm() : 8);
}
constexpr int kSpmvThreads = 256;

// Host arrays of the caller straight to / from the copy engine.  A copy from
// pageable memory returns once the source has been taken (the caller may
// reuse it); the copy back is waited for, pinned or not.
int h2d(help_pcg* ctx, double* dst, const double* src, size_t n) {
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    return HELP_OK;
}
int d2h(help_pcg* ctx, double* dst, const double* src, size_t n) {
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HELP_OK;
}

// The upload done by a kernel that reads the host array directly, where the
// device reaches pageable memory through the host page tables
// (ctx->host_direct): for a few hundred KB that takes ~5 us against ~15 us
// for cudaMemcpyAsync from pageable memory, and no staging.  The kernel reads
// the source after h2d_direct returns, so only calls that wait for their
// stream before returning use it (the caller's arrays stay valid for the
// duration of the call); those calls also let their last pass store its
// rows straight into the caller's output array where the rows come in index
// order (A's own CSR / CSC: a warp's stores are contiguous), and write the
// sliced layout's results (rows permuted within windows, so their stores
// would cross the host link as scattered 8-byte writes) with one coalesced
// copy kernel: (A D^-1 A^T) v on config 1 85.5 -> 74 us per call; the same
// copy kernel after config 4's A v / A^T y (row order) cost 0.97 -> 1.09 /
// 1.04 -> 1.34 ms, so those keep the direct stores.
int h2d_direct(help_pcg* ctx, double* dst, const double* src, size_t n) {
    if (!ctx->host_direct) return h2d(ctx, dst, src, n);
    CK(vec_copy(src, dst, (int64_t)n, ctx->num_sms, ctx->stream));
    return HELP_OK;
}
int read_status(help_pcg* ctx, const char* where) {
    int st = 0;
    CK(cudaMemcpyAsync(&st, &ctrl_of(ctx)->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st != 0) {
        CK(cudaMemsetAsync(&ctrl_of(ctx)->status, 0, sizeof(int), ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return fail(ctx, st == kStatusTimeout ? HELP_E_TIMEOUT : HELP_E_NUMERIC,
                    std::string(where) + (st == kStatusTimeout ? ": device wait timed out" : ": numerical failure"));
    }
    return HELP_OK;
}

// ---------------------------------------------------------------- CG runs

struct CgResult {
    long long iterations = 0;
    double rr0 = 0, rr = 0;
    int converged = 0;
    int status = 0;
};

// FP64-equivalent work of one CG iteration: below kClusterWorkMax one
// thread-block cluster runs the iterations faster than six launches per
// iteration over the whole GPU.
int64_t cluster_work(const help_pcg* ctx) {
    return 2 * (ctx->nnz + ctx->nnz_c) + 8 * (int64_t)ctx->m + (int64_t)ctx->k * ctx->k;
}

// Cluster size of the shared-memory-resident CG for this precision, or 0
// when it does not apply: vectors too large, too many pivots, or a row of B
// or B^T longer than 32 G nonzeros (those rows need a warp or CTA each).
int resident_fits(const help_pcg* ctx, bool f32) {
    const int slot = f32 ? 1 : 0;
    if (ctx->resident_cs[slot] <= 0) return 0;
    const RowSplit& a = f32 ? ctx->pl_csr.s32 : ctx->pl_csr.s64;
    const RowSplit& b = f32 ? ctx->pl_csc.s32 : ctx->pl_csc.s64;
    if (a.n_med + a.n_long + b.n_med + b.n_long != 0) return 0;
    return ctx->resident_cs[slot];
}

// Whether an FP32 CG run would take the multi-kernel graph path, the one
// that streams the matrix from HBM: on the resident and cluster paths an
// iteration is bound by barrier and dependent-load latency, and FP32 saves
// nothing there (measured: 12.0 against 11.4 us per iteration on config 0).
bool fp32_on_graph(const help_pcg* ctx) {
    const int p = ctx->opt.cg_path;
    if (resident_fits(ctx, true) > 0 && (p == 0 || p == 3)) return false;
    const int cs = ctx->cluster_cs[1];
    if (cs > 0 && p == 2) return false;
    if (cs > 0 && (p == 0 || p == 3) && cluster_work(ctx) <= kClusterWorkMax) return false;
    return true;
}

int finish_pcg(help_pcg* ctx, bool f32, const CgScalars* h, CgResult* res) {
    CK(cudaEventSynchronize(ctx->ev1));
    float kms = 0.f;
    CK(cudaEventElapsedTime(&kms, ctx->ev0, ctx->ev1));
    ctx->solve_kernel_ms += kms;
    ctx->solve_launches += 1;
    if (f32) ctx->solve_iters_f32 += h->it;
    res->iterations = h->it;
    res->rr0 = h->rr0;
    res->rr = h->rr;
    res->converged = (h->done == 1);
    res->status = h->status;
    if (h->done == 3) return fail(ctx, HELP_E_NUMERIC, "pcg: breakdown (non-positive curvature or NaN)");
    return HELP_OK;
}

template <class V>
int run_pcg(help_pcg* ctx, V* x, V* r0, double tol, long long max_iter, int precond_only, CgResult* res) {
    const bool f32 = std::is_same<V, float>::value;
    const int slot = f32 ? 1 : 0;
    const int nb = ctx->cg_blocks;
    // zero every byte, padding included: the graph below is re-captured when
    // these bytes change
    CgArgs<V> A;
    std::memset(static_cast<void*>(&A), 0, sizeof(A));
    A.m = ctx->m;
    A.n = ctx->n;
    A.k = ctx->k;
    A.csr = view<V>(ctx->pl_csr, ctx->rp, ctx->ci, f32 ? ctx->bv32 : ctx->bv, true);
    A.csc = view<V>(ctx->pl_csc, ctx->cp, ctx->ri, f32 ? ctx->bvT32 : ctx->bvT, true);
    A.c = view<V>(ctx->pl_c, ctx->c_rp, ctx->c_ci, f32 ? ctx->c_v32 : ctx->c_v);
    A.ct = view<V>(ctx->pl_ct, ctx->ct_rp, ctx->ct_ci, f32 ? ctx->ct_v32 : ctx->ct_v);
    A.piv = ctx->piv.as<int>();
    A.pivpos = ctx->pivpos.as<int>();
    A.W = ctx->W.as<double>();
    A.dsinv = f32 ? (const V*)ctx->dsinv32.p : (const V*)ctx->dsinv.p;
    A.delta = ctx->opt.delta;
    A.x = x;
    A.r0 = r0;
    A.r1 = f32 ? (V*)ctx->r132.p : (V*)ctx->r1.p;
    A.z = f32 ? (V*)ctx->z32.p : (V*)ctx->z.p;
    A.p0 = f32 ? (V*)ctx->p032.p : (V*)ctx->p0.p;
    A.p1 = f32 ? (V*)ctx->p132.p : (V*)ctx->p1.p;
    A.q = f32 ? (V*)ctx->q32.p : (V*)ctx->q.p;
    A.t = f32 ? (V*)ctx->t32.p : (V*)ctx->t.p;
    A.a = ctx->a.as<double>();
    A.w = ctx->w.as<double>();
    double* part = ctx->cg_part.as<double>();
    A.part_rr = part;
    A.part_rz = part + nb;
    A.part_aw = part + 2 * nb;
    A.part_pq = part + 3 * nb;
    A.precond_only = precond_only;
    A.stage_a = (A.k > 0 && A.k <= 8192 && ctx->nnz_c >= 4 * (int64_t)nb * A.k) ? 1 : 0;
    DevCtrl* c = ctrl_of(ctx);
    A.sc = &c->cg;
    // scalars the host sets: tolerance and cap (everything else the init kernel writes)
    CgScalars* h = ctx->h_sc;
    std::memset(h, 0, sizeof(*h));
    h->tol2 = tol * tol;
    h->max_iter = max_iter;
    CK(cudaMemcpyAsync(&c->cg, h, sizeof(CgScalars), cudaMemcpyHostToDevice, ctx->stream));
    const int cs = ctx->cluster_cs[slot];
    bool cluster = false, resident = false;
    if (!precond_only) {
        const int rcs = resident_fits(ctx, f32);
        if (rcs > 0 && (ctx->opt.cg_path == 0 || ctx->opt.cg_path == 3)) resident = true;
        else if (cs > 0 && ctx->opt.cg_path == 2) cluster = true;
        else if (cs > 0 && (ctx->opt.cg_path == 0 || ctx->opt.cg_path == 3))
            cluster = cluster_work(ctx) <= kClusterWorkMax;
    }
    ctx->stats.cg_path_used = resident ? 3 : cluster ? 2 : 1;
    if (resident) {
        const int rcs = ctx->resident_cs[slot];
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        CK(cg_launch_init<V>(A, nb, ctx->stream));
        int per = 64;
        for (;;) {
            CK(cg_launch_resident<V>(A, ctx->resident_layout[slot], rcs, per, ctx->stream));
            CK(cudaMemcpyAsync(h, &c->cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            if (h->done != 0) break;
            per = std::min(per * 2, 4096);
        }
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        return finish_pcg(ctx, f32, h, res);
    }
    if (cluster) {
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        CK(cg_launch_init<V>(A, nb, ctx->stream));
        int per = 64;
        for (;;) {
            CK(cg_launch_cluster<V>(A, cs, per, ctx->stream));
            CK(cudaMemcpyAsync(h, &c->cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            if (h->done != 0) break;
            per = std::min(per * 2, 4096);
        }
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        return finish_pcg(ctx, f32, h, res);
    }
    // (re)capture the per-iteration graph when the arguments changed
    std::vector<unsigned char>& key = ctx->graph_args[slot];
    if (!ctx->graph_exec[slot] || key.size() != sizeof(A) || std::memcmp(key.data(), &A, sizeof(A)) != 0) {
        if (ctx->graph_exec[slot]) {
            cudaGraphExecDestroy(ctx->graph_exec[slot]);
            ctx->graph_exec[slot] = nullptr;
        }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaSuccess;
        for (int u = 0; u < kGraphIters && ce == cudaSuccess; ++u) ce = cg_launch_iteration<V>(A, nb, ctx->stream);
        cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
        CK(ce);
        CK(ee);
        ee = cudaGraphInstantiate(&ctx->graph_exec[slot], g, 0);
        cudaGraphDestroy(g);
        CK(ee);
        key.assign((const unsigned char*)&A, (const unsigned char*)&A + sizeof(A));
    }
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    CK(cg_launch_init<V>(A, nb, ctx->stream));
    for (;;) {
        CK(cudaGraphLaunch(ctx->graph_exec[slot], ctx->stream));
        CK(cudaMemcpyAsync(h, &c->cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (h->done != 0 || precond_only) break;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    return finish_pcg(ctx, f32, h, res);
}

// res = rhs - G x  (FP64), returns ||res||^2 in *rr (host)
int residual_f64(help_pcg* ctx, const double* x, const double* rhs, double* res, double* rr) {
    CK(spmv_launch<double>(kEpiStore, view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT, true), x, ctx->t.as<double>(),
                           nullptr, nullptr, nullptr, 0.0, spmv_blocks(ctx), kSpmvThreads, ctx->stream));
    CK(spmv_launch<double>(kEpiResid, view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv, true), ctx->t.as<double>(), res,
                           rhs, x, nullptr, ctx->opt.delta, spmv_blocks(ctx), kSpmvThreads, ctx->stream));
    if (rr) {
        double* part = ctx->partials.as<double>() + 4096;
        CK(vec_sumsq(res, ctx->m, part, part + 2048, ctx->stream));
        CK(cudaMemcpyAsync(rr, part + 2048, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return HELP_OK;
}

int sumsq_host(help_pcg* ctx, const double* v, int64_t n, double* out) {
    double* part = ctx->partials.as<double>() + 4096;
    CK(vec_sumsq(v, n, part, part + 2048, ctx->stream));
    CK(cudaMemcpyAsync(out, part + 2048, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HELP_OK;
}

// Solve G x = rhs on the device; x holds the start (zero unless warm).
int normal_solve(help_pcg* ctx, const double* rhs, double* x, bool warm, long long* iters_out, int* outer_out,
                 int* fell_back, int* converged_out) {
    const int m = ctx->m;
    long long iters = 0;
    int rc;
    *fell_back = 0;
    *outer_out = 0;
    double* r = ctx->r0.as<double>();
    double rhs2 = 0.0;
    rc = sumsq_host(ctx, rhs, m, &rhs2);
    if (rc) return rc;
    if (ctx->opt.precision == HELP_PREC_FP64) {
        CgResult res;
        double tol = ctx->opt.cg_tol;
        if (warm) {
            double rr = 0.0;
            rc = residual_f64(ctx, x, rhs, r, &rr);
            if (rc) return rc;
            // keep the reference's target ||r|| < tol * ||rhs|| relative to the cold start
            tol = (rr > 0.0) ? ctx->opt.cg_tol * std::sqrt(rhs2 / rr) : 1.0;
        } else {
            CK(cudaMemcpyAsync(r, rhs, sizeof(double) * m, cudaMemcpyDeviceToDevice, ctx->stream));
            CK(vec_fill(x, 0.0, m, ctx->stream));
        }
        rc = run_pcg<double>(ctx, x, r, tol, ctx->opt.cg_max_iter, 0, &res);
        if (rc) return rc;
        *iters_out = res.iterations;
        *converged_out = res.converged;
        return HELP_OK;
    }
    // Mixed precision: FP32 CG corrections inside FP64 iterative refinement,
    // where FP32 can pay -- chosen up front, per renew: the CG runs on the
    // bandwidth-bound graph path, and max(d) / min(d) is at most
    // mixed_max_d_spread (the FP32 operator is off by ~1e-7 relative, so
    // FP32 CG stops converging once the normal equations' conditioning,
    // which follows the spread of d, passes ~1e7-1e8).  Otherwise, and once
    // FP32 corrections stagnated in this context (interior-point iterates
    // only get worse conditioned), plain FP64 PCG to the same FP64 target.
    if (!warm) CK(vec_fill(x, 0.0, m, ctx->stream));
    const bool use_fp32 = fp32_on_graph(ctx) && ctx->d_spread <= ctx->opt.mixed_max_d_spread && !ctx->fp32_stagnated;
    ctx->stats.fp32_chosen = use_fp32 ? 1 : 0;
    double rr = 0.0;
    rc = residual_f64(ctx, x, rhs, r, &rr);
    if (rc) return rc;
    const double target2 = ctx->opt.ir_tol * ctx->opt.ir_tol * rhs2;
    int outer = 0;
    bool ok = (rr <= target2) || rhs2 == 0.0;
    double prev = rr;
    while (!ok && use_fp32 && outer < ctx->opt.ir_max_outer) {
        // scale the residual to unit norm before narrowing to FP32
        const double scale = std::sqrt(rr);
        CK(vec_to_f32_scaled(r, 1.0 / scale, ctx->r032.as<float>(), m, ctx->stream));
        CgResult res;
        CK(vec_fill_f32(ctx->x32.as<float>(), 0.0f, m, ctx->stream));
        rc = run_pcg<float>(ctx, ctx->x32.as<float>(), ctx->r032.as<float>(), ctx->opt.inner_tol,
                            ctx->opt.inner_max_iter, 0, &res);
        if (rc) return rc;
        iters += res.iterations;
        CK(vec_add_f32_scaled(x, ctx->x32.as<float>(), scale, m, ctx->stream));
        rc = residual_f64(ctx, x, rhs, r, &rr);
        if (rc) return rc;
        ++outer;
        ok = (rr <= target2);
        if (!ok && !(rr < 0.25 * prev)) {  // stagnation: FP32 corrections no longer help
            ctx->fp32_stagnated = true;
            break;
        }
        prev = rr;
    }
    *outer_out = outer;
    if (!ok && (!use_fp32 || ctx->opt.fallback)) {  // FP64 chosen up front, or the mixed form's FP64 finish
        CgResult res;
        const double tol = (rr > 0.0) ? ctx->opt.ir_tol * std::sqrt(rhs2 / rr) : 1.0;
        rc = run_pcg<double>(ctx, x, r, std::min(tol, 1.0), ctx->opt.cg_max_iter, 0, &res);
        if (rc) return rc;
        iters += res.iterations;
        *fell_back = use_fp32 ? 1 : 0;
        ok = res.converged != 0;
    }
    *iters_out = iters;
    *converged_out = ok ? 1 : 0;
    return HELP_OK;
}

int alloc_vectors(help_pcg* ctx) {
    const size_t m = ctx->m, n = ctx->n;
    const size_t mn = std::max(m, n);
    CK(ctx->x.ensure(8 * m));
    CK(ctx->r0.ensure(8 * m));
    CK(ctx->r1.ensure(8 * m));
    CK(ctx->z.ensure(8 * m));
    CK(ctx->p0.ensure(8 * m));
    CK(ctx->p1.ensure(8 * m));
    CK(ctx->q.ensure(8 * m));
    CK(ctx->t.ensure(8 * n));
    CK(ctx->u.ensure(8 * n));
    CK(ctx->rhs.ensure(8 * m));
    CK(ctx->b1.ensure(8 * n));
    CK(ctx->b2.ensure(8 * m));
    CK(ctx->x1.ensure(8 * n));
    CK(ctx->x2.ensure(8 * mn));
    CK(ctx->res.ensure(8 * mn));
    CK(ctx->xacc.ensure(8 * mn));
    CK(ctx->d.ensure(8 * n));
    CK(ctx->s.ensure(8 * n));
    CK(ctx->diag.ensure(8 * m));
    CK(ctx->dsinv.ensure(8 * m));
    CK(ctx->piv.ensure(4 * m));
    CK(ctx->pivpos.ensure(4 * m));
    CK(ctx->keys.ensure(8 * m));
    CK(ctx->hist.ensure(4 * kTopkBins));
    CK(ctx->flags.ensure(4 * 3 * mn + 64));
    CK(ctx->scan_tmp.ensure(4 * scan_tmp_elems((int64_t)std::max<size_t>(mn + 1, 1u << 20) * 4)));
    CK(ctx->cr_cnt.ensure(4 * (mn + 1)));
    CK(ctx->bp_ptr.ensure(4 * (n + 1)));
    CK(ctx->c_rp.ensure(4 * (m + 1)));
    if (ctx->opt.precision == HELP_PREC_MIXED) {
        CK(ctx->x32.ensure(4 * m));
        CK(ctx->r032.ensure(4 * m));
        CK(ctx->r132.ensure(4 * m));
        CK(ctx->z32.ensure(4 * m));
        CK(ctx->p032.ensure(4 * m));
        CK(ctx->p132.ensure(4 * m));
        CK(ctx->q32.ensure(4 * m));
        CK(ctx->t32.ensure(4 * n));
        CK(ctx->dsinv32.ensure(4 * m));
    }
    return HELP_OK;
}

void release_all(help_pcg* ctx) {
    DevMem* bufs[] = {&ctx->rp,     &ctx->ci,    &ctx->av,     &ctx->cp,     &ctx->ri,    &ctx->avT,   &ctx->bv,
                      &ctx->bvT,    &ctx->bv32,  &ctx->bvT32,  &ctx->d,      &ctx->s,     &ctx->diag,  &ctx->dsinv,
                      &ctx->dsinv32, &ctx->piv,  &ctx->pivpos, &ctx->keys,   &ctx->hist,  &ctx->flags, &ctx->scan_tmp,
                      &ctx->bp_ptr, &ctx->bp_c,  &ctx->bp_v,   &ctx->cr_cnt, &ctx->c_rp,  &ctx->c_ci,  &ctx->c_v,
                      &ctx->c_v32,  &ctx->ct_rp, &ctx->ct_ci,  &ctx->ct_v,   &ctx->ct_v32, &ctx->ct_blk, &ctx->g11,
                      &ctx->W,      &ctx->lwork, &ctx->x,      &ctx->r0,     &ctx->r1,    &ctx->z,     &ctx->p0,
                      &ctx->p1,     &ctx->q,     &ctx->t,      &ctx->a,      &ctx->w,     &ctx->x32,   &ctx->r032,
                      &ctx->r132,   &ctx->z32,   &ctx->p032,   &ctx->p132,   &ctx->q32,   &ctx->t32,   &ctx->u,
                      &ctx->rhs,    &ctx->b1,    &ctx->b2,     &ctx->x1,     &ctx->x2,    &ctx->res,   &ctx->xacc,
                      &ctx->adat_tmp};
    for (DevMem* b : bufs) b->release();
    ctx->cg_part.release();
    for (int s = 0; s < 2; ++s) {
        if (ctx->graph_exec[s]) cudaGraphExecDestroy(ctx->graph_exec[s]);
        ctx->graph_exec[s] = nullptr;
        ctx->graph_args[s].clear();
    }
    RowPlan* plans[] = {&ctx->pl_csr, &ctx->pl_csc, &ctx->pl_c, &ctx->pl_ct};
    for (RowPlan* p : plans) {
        for (RowSplit* s : {&p->s64, &p->s32}) {
            for (DevMem* d : {&s->med, &s->lng, &s->seg, &s->lnseg, &s->lbase, &s->tickets, &s->parts, &s->sorder})
                d->release();
            s->n_med = s->n_long = s->n_seg = s->n_short = 0;
        }
        p->rows = 0;
    }
}

int read_int(help_pcg* ctx, const int* dev, int* out) {
    CK(cudaMemcpyAsync(out, dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HELP_OK;
}

// Features of the current renew for solve slot `slot` into X (BF16 [m][16],
// the attached model's normalisation) or, X null, raw into R.  D_S is the
// uncorrected one.
int learned_features(help_pcg* ctx, int slot, __nv_bfloat16* X, float* R) {
    const int prev = ctx->x2_cur ^ 1;
    const double* xprev = ctx->x2_have[prev][slot] ? ctx->x2h[prev][slot].as<double>() : nullptr;
    double* part = ctx->partials.as<double>() + 4096;
    if (xprev) CK(vec_sumsq(xprev, ctx->m, part, part + 2048, ctx->stream));
    const double* dsinv = ctx->mlp_active ? ctx->dsinv_plain.as<double>() : ctx->dsinv.as<double>();
    CK(mlp_features(ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->d.as<double>(), ctx->diag.as<double>(), dsinv,
                    ctx->pivpos.as<int>(), xprev, part + 2048, ctx->have_dprev ? ctx->d_prev.as<double>() : nullptr,
                    ctx->m, ctx->mlp ? help_mlp_device_weights(ctx->mlp) : nullptr, X, R, ctx->stream));
    return HELP_OK;
}

// Features of `slot` and the model's outputs for them into mlp_out.
int learned_forward(help_pcg* ctx, int slot) {
    const int m = ctx->m;
    CK(ctx->mlp_x.ensure(2 * (size_t)HELP_MLP_IN * m));
    CK(ctx->mlp_out.ensure(sizeof(float) * HELP_MLP_OUT * (size_t)m));
    int rc = learned_features(ctx, slot, ctx->mlp_x.as<__nv_bfloat16>(), nullptr);
    if (rc) return rc;
    CK(mlp_forward(ctx->mlp_x.as<__nv_bfloat16>(), m, help_mlp_device_weights(ctx->mlp), ctx->mlp_out.as<float>(),
                   nullptr, nullptr, ctx->num_sms, ctx->stream));
    return HELP_OK;
}

// After a renew with a model attached: features, forward, corrected D_S^-1
// (the plain one kept for the fallback).
int learned_renew(help_pcg* ctx) {
    const int m = ctx->m;
    CK(ctx->dsinv_plain.ensure(8 * (size_t)m));
    int rc = learned_forward(ctx, 0);  // the correction is slot 0's output
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->dsinv_plain.p, ctx->dsinv.p, 8 * (size_t)m, cudaMemcpyDeviceToDevice, ctx->stream));
    const bool mixed = ctx->opt.precision == HELP_PREC_MIXED;
    CK(mlp_apply_diag(ctx->mlp_out.as<float>(), ctx->pivpos.as<int>(), ctx->dsinv.as<double>(),
                      mixed ? ctx->dsinv32.as<float>() : nullptr, m, ctx->stream));
    ctx->mlp_active = true;
    return HELP_OK;
}

// Undo the model's correction for the rest of this renew.
int learned_restore(help_pcg* ctx) {
    const int m = ctx->m;
    CK(cudaMemcpyAsync(ctx->dsinv.p, ctx->dsinv_plain.p, 8 * (size_t)m, cudaMemcpyDeviceToDevice, ctx->stream));
    if (ctx->opt.precision == HELP_PREC_MIXED)
        CK(vals_to_f32(ctx->dsinv.as<double>(), ctx->dsinv32.as<float>(), m, ctx->stream));
    ctx->mlp_active = false;
    return HELP_OK;
}

// x = alpha v, v = out[:,1] .* x_2 of this slot in the previous renew, alpha
// minimising the G-norm error along v.  *used = false when there is no
// previous solution or v is zero.
int learned_warm_start(help_pcg* ctx, int slot, bool* used) {
    *used = false;
    const int prev = ctx->x2_cur ^ 1;
    if (!ctx->x2_have[prev][slot]) return HELP_OK;
    const int m = ctx->m;
    if (slot > 0) {  // this slot's own features (slot 0's came with the renew)
        const int rc = learned_forward(ctx, slot);
        if (rc) return rc;
    }
    double* x = ctx->x.as<double>();
    double* gv = ctx->res.as<double>();
    CK(mlp_warm_vector(ctx->mlp_out.as<float>(), ctx->x2h[prev][slot].as<double>(), x, m, ctx->stream));
    CK(spmv_launch<double>(kEpiStore, view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT, true), x, ctx->t.as<double>(),
                           nullptr, nullptr, nullptr, 0.0, spmv_blocks(ctx), kSpmvThreads, ctx->stream));
    CK(spmv_launch<double>(kEpiAddDelta, view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv, true), ctx->t.as<double>(), gv,
                           x, nullptr, nullptr, ctx->opt.delta, spmv_blocks(ctx), kSpmvThreads, ctx->stream));
    double* part = ctx->partials.as<double>() + 4096;
    CK(vec_dot(x, ctx->rhs.as<double>(), m, part, part + 2049, ctx->stream));
    CK(vec_dot(x, gv, m, part, part + 2050, ctx->stream));
    double h[2] = {0.0, 0.0};
    CK(cudaMemcpyAsync(h, part + 2049, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const double alpha = h[1] > 0.0 ? h[0] / h[1] : 0.0;
    if (!(alpha == alpha) || alpha == 0.0 || std::isinf(alpha)) return HELP_OK;
    CK(vec_scale(x, alpha, m, ctx->stream));
    *used = true;
    return HELP_OK;
}

int renew_impl(help_pcg* ctx, const double* d_host) {
    const double t0 = now_ms();
    const int m = ctx->m, n = ctx->n;
    const bool mixed = ctx->opt.precision == HELP_PREC_MIXED;
    DevCtrl* c = ctrl_of(ctx);
    // the learned part's features compare d with the previous renew's
    ctx->have_dprev = false;
    if (ctx->mlp && ctx->renewed) {
        CK(ctx->d_prev.ensure(8 * (size_t)n));
        CK(cudaMemcpyAsync(ctx->d_prev.p, ctx->d.p, 8 * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
        ctx->have_dprev = true;
    }
    int rc = h2d(ctx, ctx->d.as<double>(), d_host, n);
    if (rc) return rc;
    CK(renew_inv_sqrt(ctx->d.as<double>(), ctx->s.as<double>(), n, &c->status, ctx->stream));
    rc = read_status(ctx, "renew: d must be positive and finite");
    if (rc) return rc;
    CK(renew_scale_values(ctx->s.as<double>(), ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->av.as<double>(),
                          ctx->bv.as<double>(), mixed ? ctx->bv32.as<float>() : nullptr, ctx->cp.as<int>(),
                          ctx->avT.as<double>(), ctx->bvT.as<double>(), mixed ? ctx->bvT32.as<float>() : nullptr,
                          ctx->diag.as<double>(), ctx->opt.delta, m, n, ctx->nnz, &c->status, ctx->stream));
    rc = read_status(ctx, "renew: a row of A has no nonzeros, so A D^-1 A^T is singular (remove the row or set delta > 0)");
    if (rc) return rc;
    rc = refresh_sell(ctx, mixed);
    if (rc) return rc;
    // pivots
    const int k = std::max(0, std::min(ctx->opt.pivots, m));
    ctx->k = k;
    CK(topk_select(ctx->diag.as<double>(), m, k, ctx->keys.as<unsigned long long>(), ctx->hist.as<unsigned int>(),
                   ctx->flags.as<int>(), ctx->scan_tmp.as<int>(), &c->topk, &c->status, ctx->piv.as<int>(),
                   ctx->pivpos.as<int>(), ctx->stream));
    rc = read_status(ctx, "renew: diag(A D^-1 A^T) not finite");
    if (rc) return rc;
    // pivot entries per column
    int* cnt = ctx->cr_cnt.as<int>();
    CK(pivot_lists_count(ctx->cp.as<int>(), ctx->ri.as<int>(), ctx->pivpos.as<int>(), n, cnt, ctx->stream));
    CK(exclusive_scan(cnt, ctx->bp_ptr.as<int>(), n, ctx->scan_tmp.as<int>(), &c->totals[0], ctx->stream));
    int nbp = 0;
    rc = read_int(ctx, &c->totals[0], &nbp);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->bp_ptr.as<int>() + n, &c->totals[0], sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
    CK(ctx->bp_c.ensure(4 * (size_t)std::max(nbp, 1)));
    CK(ctx->bp_v.ensure(8 * (size_t)std::max(nbp, 1)));
    CK(pivot_lists_fill(ctx->cp.as<int>(), ctx->ri.as<int>(), ctx->bvT.as<double>(), ctx->pivpos.as<int>(), n,
                        ctx->bp_ptr.as<int>(), ctx->bp_c.as<int>(), ctx->bp_v.as<double>(), ctx->stream));
    // G[i, P]: counts, row pointers of C, fill (C rows and dense G11)
    CK(ctx->g11.ensure(8 * (size_t)std::max(k, 1) * std::max(k, 1)));
    CK(ctx->W.ensure(8 * (size_t)std::max(k, 1) * std::max(k, 1)));
    CK(ctx->lwork.ensure(8 * dense_work_elems(std::max(k, 1))));
    CK(ctx->a.ensure(8 * (size_t)std::max(k, 1)));
    CK(ctx->w.ensure(8 * (size_t)std::max(k, 1)));
    CK(gcols_rows(0, ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->bv.as<double>(), ctx->bp_ptr.as<int>(),
                  ctx->bp_c.as<int>(), ctx->bp_v.as<double>(), ctx->pivpos.as<int>(), m, k, ctx->opt.delta, cnt,
                  nullptr, nullptr, nullptr, nullptr, ctx->num_sms, ctx->stream));
    CK(exclusive_scan(cnt, ctx->c_rp.as<int>(), m, ctx->scan_tmp.as<int>(), &c->totals[1], ctx->stream));
    int nnzc = 0;
    rc = read_int(ctx, &c->totals[1], &nnzc);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->c_rp.as<int>() + m, &c->totals[1], sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->nnz_c = nnzc;
    CK(ctx->c_ci.ensure(4 * (size_t)std::max(nnzc, 1)));
    CK(ctx->c_v.ensure(8 * (size_t)std::max(nnzc, 1)));
    if (k > 0) CK(cudaMemsetAsync(ctx->g11.p, 0, 8 * (size_t)k * k, ctx->stream));
    CK(gcols_rows(1, ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->bv.as<double>(), ctx->bp_ptr.as<int>(),
                  ctx->bp_c.as<int>(), ctx->bp_v.as<double>(), ctx->pivpos.as<int>(), m, k, ctx->opt.delta, nullptr,
                  ctx->c_rp.as<int>(), ctx->c_ci.as<int>(), ctx->c_v.as<double>(), ctx->g11.as<double>(),
                  ctx->num_sms, ctx->stream));
    // C^T
    CK(ctx->ct_rp.ensure(4 * (size_t)(k + 1)));
    CK(ctx->ct_ci.ensure(4 * (size_t)std::max(nnzc, 1)));
    CK(ctx->ct_v.ensure(8 * (size_t)std::max(nnzc, 1)));
    if (k > 0) {
        const int nblk = (m + ct_rows_per_block() - 1) / ct_rows_per_block();
        const size_t nb = (size_t)k * nblk;
        CK(ctx->ct_blk.ensure(4 * (2 * nb + 2)));
        CK(ctx->scan_tmp.ensure(4 * std::max(scan_tmp_elems((int64_t)nb), scan_tmp_elems((int64_t)std::max(m, n) + 1))));
        int* blk_cnt = ctx->ct_blk.as<int>();
        int* blk_off = blk_cnt + nb + 1;
        CK(ct_count(ctx->c_rp.as<int>(), ctx->c_ci.as<int>(), m, k, blk_cnt, ctx->stream));
        CK(exclusive_scan(blk_cnt, blk_off, (int64_t)nb, ctx->scan_tmp.as<int>(), &c->totals[2], ctx->stream));
        CK(ct_row_ptr(blk_off, k, nblk, &c->totals[2], ctx->ct_rp.as<int>(), ctx->stream));
        CK(ct_fill(ctx->c_rp.as<int>(), ctx->c_ci.as<int>(), ctx->c_v.as<double>(), m, k, blk_off,
                   ctx->ct_ci.as<int>(), ctx->ct_v.as<double>(), ctx->stream));
    } else {
        CK(cudaMemsetAsync(ctx->ct_rp.p, 0, 4, ctx->stream));
    }
    if (mixed) {
        CK(ctx->c_v32.ensure(4 * (size_t)std::max(nnzc, 1)));
        CK(ctx->ct_v32.ensure(4 * (size_t)std::max(nnzc, 1)));
        CK(vals_to_f32(ctx->c_v.as<double>(), ctx->c_v32.as<float>(), nnzc, ctx->stream));
        CK(vals_to_f32(ctx->ct_v.as<double>(), ctx->ct_v32.as<float>(), nnzc, ctx->stream));
    }
    // plans for C and C^T
    ctx->h_tmp.resize((size_t)m + 1);
    CK(cudaMemcpyAsync(ctx->h_tmp.data(), ctx->c_rp.p, 4 * ((size_t)m + 1), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    rc = upload_plan(ctx, ctx->pl_c, ctx->h_tmp.data(), m, mixed, nullptr, kPerLaneCF64, kPerLaneCF32, kOrderWasteC);
    if (rc) return rc;
    std::vector<int32_t> ctp((size_t)k + 1, 0);
    if (k > 0) {
        CK(cudaMemcpyAsync(ctp.data(), ctx->ct_rp.p, 4 * ((size_t)k + 1), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    rc = upload_plan(ctx, ctx->pl_ct, ctp.data(), k, mixed);
    if (rc) return rc;
    // shared-memory-resident CG: layout for this renew's C (h_tmp = C's row pointers)
    ctx->resident_cs[0] = cg_resident_configure<double>(m, n, k, ctx->h_rp.data(), ctx->h_cp.data(),
                                                        ctx->h_tmp.data(), &ctx->resident_layout[0]);
    ctx->resident_cs[1] = mixed ? cg_resident_configure<float>(m, n, k, ctx->h_rp.data(), ctx->h_cp.data(),
                                                               ctx->h_tmp.data(), &ctx->resident_layout[1])
                                : 0;
    // pivot block inverse and the Schur diagonal
    CK(cudaMemsetAsync(&c->regularised, 0, sizeof(int), ctx->stream));
    if (k > 0)
        CK(dense_spd_inverse(ctx->g11.as<double>(), ctx->W.as<double>(), ctx->lwork.as<double>(), k, &c->regularised,
                             ctx->stream));
    CK(schur_diag(ctx->c_rp.as<int>(), ctx->c_ci.as<int>(), ctx->c_v.as<double>(), ctx->W.as<double>(),
                  ctx->diag.as<double>(), ctx->pivpos.as<int>(), m, k, 1.0e-14, ctx->dsinv.as<double>(),
                  mixed ? ctx->dsinv32.as<float>() : nullptr, ctx->stream));
    rc = read_int(ctx, &c->regularised, &ctx->dense_regularised);
    if (rc) return rc;
    // this renew's solves seed the next renew's warm starts
    ctx->x2_cur ^= 1;
    for (int q = 0; q < kSolveSlots; ++q) ctx->x2_have[ctx->x2_cur][q] = false;
    ctx->solve_slot = 0;
    ctx->mlp_active = false;
    if (ctx->mlp) {
        rc = learned_renew(ctx);
        if (rc) return rc;
    }
    CK(cudaGetLastError());
    ctx->renewed = true;
    ctx->have_prev_x2 = false;
    ctx->stats.renews++;
    ctx->stats.renew_ms = now_ms() - t0;
    ctx->stats.nnz_c = ctx->nnz_c;
    ctx->stats.pivots = k;
    ctx->stats.dense_regularised = ctx->dense_regularised;
    return HELP_OK;
}

}  // namespace

// ================================================================ C ABI

extern "C" {

void help_pcg_default_options(help_pcg_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->device = 0;
    o->pivots = 10;
    o->precision = HELP_PREC_FP64;
    o->cg_tol = 1e-20;
    o->cg_max_iter = 1000000;
    o->delta = 0.0;
    o->ir_tol = 1e-10;
    o->ir_max_outer = 10;
    o->inner_tol = 1e-5;
    o->inner_max_iter = 200000;
    o->warm_start = 0;
    o->fallback = 1;
    o->cg_path = 0;
    o->cap_ok = 0;
    o->mixed_max_d_spread = 1e8;
}

static int help_pcg_create_body(const help_pcg_options* opt, help_pcg** out) {
    if (!out) return HELP_E_ARG;
    *out = nullptr;
    help_pcg* ctx = new (std::nothrow) help_pcg();
    if (!ctx) return HELP_E_NOMEM;
    if (opt) ctx->opt = *opt;
    else help_pcg_default_options(&ctx->opt);
    if (ctx->opt.precision != HELP_PREC_FP64 && ctx->opt.precision != HELP_PREC_MIXED) {
        delete ctx;
        return HELP_E_ARG;
    }
    ctx->device = ctx->opt.device;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) {
        // Grace systems: kernels may read and write pageable host memory
        // directly (address translation through the host page tables)
        int pageable = 0, host_tables = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, ctx->device) == cudaSuccess &&
            cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ctx->device) ==
                cudaSuccess)
            ctx->host_direct = pageable == 1 && host_tables == 1;
        cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = ctx->ctrl.ensure(sizeof(DevCtrl));
    if (e == cudaSuccess) e = cudaMemset(ctx->ctrl.p, 0, sizeof(DevCtrl));
    if (e == cudaSuccess) e = ctx->partials.ensure(8 * (size_t)kPartElems);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_sc, sizeof(CgScalars));
    if (e != cudaSuccess) {
        release_all(ctx);
        for (cudaEvent_t ev : {ctx->ev0, ctx->ev1})
            if (ev) cudaEventDestroy(ev);
        if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return e == cudaErrorMemoryAllocation ? HELP_E_NOMEM : HELP_E_CUDA;
    }
    *out = ctx;
    return HELP_OK;
}

int help_pcg_create(const help_pcg_options* opt, help_pcg** out) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_create_body(opt, out); });
}

void help_pcg_free(help_pcg* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    help_pcg_destruct(ctx);
    ctx->ctrl.release();
    ctx->partials.release();
    for (int s = 0; s < 2; ++s)
        if (ctx->graph_exec[s]) cudaGraphExecDestroy(ctx->graph_exec[s]);
    if (ctx->h_sc) cudaFreeHost(ctx->h_sc);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static int help_pcg_construct_body(help_pcg* ctx, int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                       const double* val) {
    if (!ctx) return HELP_E_ARG;
    if (ctx->constructed) return fail(ctx, HELP_E_ARG, "construct: already constructed (call destruct first)");
    if (m <= 0 || n <= 0 || !col_ptr || !row_ind || !val) return fail(ctx, HELP_E_ARG, "construct: bad arguments");
    if (col_ptr[0] != 0) return fail(ctx, HELP_E_ARG, "construct: col_ptr[0] must be 0");
    for (int32_t j = 0; j < n; ++j)
        if (col_ptr[j + 1] < col_ptr[j]) return fail(ctx, HELP_E_ARG, "construct: col_ptr not monotone");
    const int64_t nnz = col_ptr[n];
    for (int32_t j = 0; j < n; ++j)
        for (int32_t p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
            if (row_ind[p] < 0 || row_ind[p] >= m) return fail(ctx, HELP_E_ARG, "construct: row index out of range");
            if (p > col_ptr[j] && row_ind[p] <= row_ind[p - 1])
                return fail(ctx, HELP_E_ARG, "construct: rows must be strictly increasing inside a column");
        }
    CK(cudaSetDevice(ctx->device));
    ctx->m = m;
    ctx->n = n;
    ctx->nnz = nnz;
    // CSR(A) from CSC(A) (UsePCG_CPU.cpp:53-66 builds it from the row lists)
    ctx->h_cp.assign(col_ptr, col_ptr + n + 1);
    ctx->h_rp.assign((size_t)m + 1, 0);
    std::vector<int32_t> ci((size_t)std::max<int64_t>(nnz, 1));
    std::vector<double> av((size_t)std::max<int64_t>(nnz, 1));
    for (int64_t p = 0; p < nnz; ++p) ctx->h_rp[row_ind[p] + 1]++;
    for (int32_t i = 0; i < m; ++i) ctx->h_rp[i + 1] += ctx->h_rp[i];
    {
        std::vector<int32_t> fill(ctx->h_rp.begin(), ctx->h_rp.end() - 1);
        for (int32_t j = 0; j < n; ++j)
            for (int32_t p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
                const int32_t q = fill[row_ind[p]]++;
                ci[q] = j;
                av[q] = val[p];
            }
    }
    CK(ctx->rp.ensure(4 * ((size_t)m + 1)));
    CK(ctx->ci.ensure(4 * (size_t)nnz));
    CK(ctx->av.ensure(8 * (size_t)nnz));
    CK(ctx->cp.ensure(4 * ((size_t)n + 1)));
    CK(ctx->ri.ensure(4 * (size_t)nnz));
    CK(ctx->avT.ensure(8 * (size_t)nnz));
    CK(ctx->bv.ensure(8 * (size_t)nnz));
    CK(ctx->bvT.ensure(8 * (size_t)nnz));
    const bool mixed = ctx->opt.precision == HELP_PREC_MIXED;
    if (mixed) {
        CK(ctx->bv32.ensure(4 * (size_t)nnz));
        CK(ctx->bvT32.ensure(4 * (size_t)nnz));
    }
    CK(cudaMemcpyAsync(ctx->rp.p, ctx->h_rp.data(), 4 * ((size_t)m + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->ci.p, ci.data(), 4 * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->av.p, av.data(), 8 * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->cp.p, col_ptr, 4 * ((size_t)n + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->ri.p, row_ind, 4 * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->avT.p, val, 8 * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int rc = upload_plan(ctx, ctx->pl_csr, ctx->h_rp.data(), m, mixed, ci.data());
    if (!rc) rc = upload_plan(ctx, ctx->pl_csc, ctx->h_cp.data(), n, mixed, row_ind);
    if (!rc) rc = alloc_vectors(ctx);
    if (rc) return rc;
    // CG kernels: grid-stride, grid sized to the work (small problems pay
    // less for the per-block partial sums), at most one wave of resident
    // CTAs of the graph kernels (6 per SM at their 40 registers; 8 per SM,
    // a partial second wave, measured per FP64 iteration: config 3 100.1 ->
    // 89.6 us, config 4 2,230 -> 2,047 us, config 2 365 -> 376 us)
    {
        const int64_t work = std::max<int64_t>(nnz, 32 * (int64_t)std::max(m, n));
        const int64_t nb = (work + 16383) / 16384;
        ctx->cg_blocks =
            (int)std::max<int64_t>(8, std::min<int64_t>(nb, (int64_t)ctx->num_sms * cg_blocks_per_sm()));
    }
    CK(ctx->cg_part.ensure(sizeof(double) * 4 * (size_t)ctx->cg_blocks));
    CK(cg_configure<double>(std::max(ctx->opt.pivots, 1)));
    if (mixed) CK(cg_configure<float>(std::max(ctx->opt.pivots, 1)));
    ctx->cluster_cs[0] = cg_cluster_configure<double>(std::max(ctx->opt.pivots, 1));
    ctx->cluster_cs[1] = mixed ? cg_cluster_configure<float>(std::max(ctx->opt.pivots, 1)) : 0;
    ctx->stats.cluster_ctas = ctx->cluster_cs[0];
    cudaGetLastError();
    ctx->constructed = true;
    ctx->renewed = false;
    return HELP_OK;
}

int help_pcg_construct(help_pcg* ctx, int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                       const double* val) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_construct_body(ctx, m, n, col_ptr, row_ind, val); });
}

static int help_pcg_destruct_body(help_pcg* ctx) {
    if (!ctx) return HELP_E_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    release_all(ctx);
    ctx->constructed = false;
    ctx->renewed = false;
    ctx->last_d = nullptr;
    ctx->m = ctx->n = 0;
    ctx->nnz = 0;
    return HELP_OK;
}

int help_pcg_destruct(help_pcg* ctx) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_destruct_body(ctx); });
}

static int help_pcg_renew_body(help_pcg* ctx, const double* d) {
    if (!ctx || !d) return HELP_E_ARG;
    if (!ctx->constructed) return fail(ctx, HELP_E_ARG, "renew: construct first");
    CK(cudaSetDevice(ctx->device));
    int rc = renew_impl(ctx, d);
    if (rc) {
        ctx->renewed = false;
        return rc;
    }
    ctx->last_d = d;
    // spread of d for the mixed form's choice (renew_impl has checked that
    // every d is positive and finite)
    double dmin = d[0], dmax = d[0];
    for (int j = 1; j < ctx->n; ++j) {
        dmin = std::min(dmin, d[j]);
        dmax = std::max(dmax, d[j]);
    }
    ctx->d_spread = dmax / dmin;
    ctx->stats.d_spread = ctx->d_spread;
    return HELP_OK;
}

int help_pcg_renew(help_pcg* ctx, const double* d) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_renew_body(ctx, d); });
}

static int help_pcg_solve_body(help_pcg* ctx, const double* d, const double* b_1, const double* b_2, double* x_1,
                   double* x_2) {
    if (!ctx || !d || !b_1 || !b_2 || !x_1 || !x_2) return HELP_E_ARG;
    if (!ctx->constructed) return fail(ctx, HELP_E_ARG, "solve: construct first");
    CK(cudaSetDevice(ctx->device));
    int rc;
    if (!ctx->renewed || d != ctx->last_d) {
        rc = help_pcg_renew(ctx, d);
        if (rc) return rc;
    }
    const double t0 = now_ms();
    const int m = ctx->m, n = ctx->n;
    ctx->solve_kernel_ms = 0;
    ctx->solve_iters_f32 = 0;
    ctx->solve_launches = 0;
    rc = h2d(ctx, ctx->b1.as<double>(), b_1, n);
    if (!rc) rc = h2d(ctx, ctx->b2.as<double>(), b_2, m);
    if (rc) return rc;
    // u = D^-1/2 b_1 ;  rhs = B u - b_2 = A D^-1 b_1 - b_2   (UsePCG_CPU.cpp:103-112)
    CK(vec_scale_mul(ctx->s.as<double>(), ctx->b1.as<double>(), ctx->u.as<double>(), n, ctx->stream));
    CK(spmv_launch<double>(kEpiRhs, view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv, true), ctx->u.as<double>(),
                           ctx->rhs.as<double>(), ctx->b2.as<double>(), nullptr, nullptr, 0.0, spmv_blocks(ctx),
                           kSpmvThreads, ctx->stream));
    // x_2 (UsePCG_CPU.cpp:154-166)
    const int slot = ctx->solve_slot < ctx->slot_map_n ? ctx->slot_map[ctx->solve_slot]
                                                       : std::min(ctx->solve_slot, kSolveSlots - 1);
    bool warm = ctx->opt.warm_start && ctx->have_prev_x2;
    bool learned_warm = false;
    if (ctx->mlp_active) {
        rc = learned_warm_start(ctx, slot, &learned_warm);
        if (rc) return rc;
        warm = learned_warm;
    }
    const bool learned = ctx->mlp_active;
    long long iters = 0;
    int outer = 0, fell_back = 0, converged = 0;
    rc = normal_solve(ctx, ctx->rhs.as<double>(), ctx->x.as<double>(), warm, &iters, &outer, &fell_back, &converged);
    if (rc) return rc;
    // true FP64 residual of the normal equations, reported with the solve
    double rr = 0.0, rhs2 = 0.0;
    rc = residual_f64(ctx, ctx->x.as<double>(), ctx->rhs.as<double>(), ctx->res.as<double>(), &rr);
    if (!rc) rc = sumsq_host(ctx, ctx->rhs.as<double>(), m, &rhs2);
    if (rc) return rc;
    if (learned) {
        // the plain preconditioner is the model's fallback: redo cold and uncorrected
        // on an iteration cap or a failed FP64 residual check
        const double rel = rhs2 > 0.0 ? std::sqrt(rr / rhs2) : std::sqrt(rr);
        if (!converged || !(rel <= std::max(1e-6, 100.0 * ctx->opt.cg_tol))) {
            rc = learned_restore(ctx);
            if (rc) return rc;
            long long it2 = 0;
            int outer2 = 0, fb2 = 0;
            rc = normal_solve(ctx, ctx->rhs.as<double>(), ctx->x.as<double>(), false, &it2, &outer2, &fb2, &converged);
            if (rc) return rc;
            iters += it2;
            outer += outer2;
            fell_back = 1;
            learned_warm = false;
            ctx->stats.learned_fallbacks++;
            rc = residual_f64(ctx, ctx->x.as<double>(), ctx->rhs.as<double>(), ctx->res.as<double>(), &rr);
            if (rc) return rc;
        }
    }
    if (ctx->mlp) {
        CK(ctx->x2h[ctx->x2_cur][slot].ensure(8 * (size_t)m));
        CK(cudaMemcpyAsync(ctx->x2h[ctx->x2_cur][slot].p, ctx->x.p, 8 * (size_t)m, cudaMemcpyDeviceToDevice,
                           ctx->stream));
        ctx->x2_have[ctx->x2_cur][slot] = true;
    }
    ctx->solve_slot++;
    ctx->stats.learned_warm = learned_warm ? 1 : 0;
    // x_1 = D^-1 (b_1 - A^T x_2) = D^-1/2 (u - B^T x_2)   (UsePCG_CPU.cpp:171-177)
    CK(spmv_launch<double>(kEpiBacksub, view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT, true), ctx->x.as<double>(),
                           ctx->x1.as<double>(), ctx->u.as<double>(), nullptr, ctx->s.as<double>(), 0.0,
                           spmv_blocks(ctx), kSpmvThreads, ctx->stream));
    rc = d2h(ctx, x_1, ctx->x1.as<double>(), n);
    if (!rc) rc = d2h(ctx, x_2, ctx->x.as<double>(), m);
    if (rc) return rc;
    ctx->have_prev_x2 = true;
    ctx->stats.cg_iterations = iters;
    ctx->stats.cg_iterations_total += iters;
    ctx->stats.ir_outer = outer;
    ctx->stats.fell_back = fell_back;
    ctx->stats.converged = converged;
    ctx->stats.rel_residual = rhs2 > 0.0 ? std::sqrt(rr / rhs2) : std::sqrt(rr);
    ctx->stats.solve_ms = now_ms() - t0;
    ctx->stats.solves++;
    ctx->stats.cg_kernel_ms = ctx->solve_kernel_ms;
    ctx->stats.cg_kernel_ms_total += ctx->solve_kernel_ms;
    ctx->stats.cg_iterations_fp32 = ctx->solve_iters_f32;
    ctx->stats.cg_launches = ctx->solve_launches;
    if (!converged && !ctx->opt.cap_ok)
        return fail(ctx, HELP_E_NOT_CONVERGED, "solve: CG stopped at its iteration cap before cg_tol");
    return HELP_OK;
}

int help_pcg_solve(help_pcg* ctx, const double* d, const double* b_1, const double* b_2, double* x_1,
                   double* x_2) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_solve_body(ctx, d, b_1, b_2, x_1, x_2); });
}

int help_pcg_get_stats(const help_pcg* ctx, help_pcg_stats* out) {
    if (!ctx || !out) return HELP_E_ARG;
    *out = ctx->stats;
    return HELP_OK;
}

const char* help_pcg_last_error(const help_pcg* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

static int help_pcg_matvec_dev_body(help_pcg* ctx, int32_t op, int32_t fp32, const void* x, void* y, void* stream) {
    if (!ctx || !x || !y) return HELP_E_ARG;
    if (!ctx->constructed) return fail(ctx, HELP_E_ARG, "matvec: construct first");
    if ((op >= HELP_OP_ADAT || fp32) && !ctx->renewed) return fail(ctx, HELP_E_ARG, "matvec: renew first");
    if (fp32 && ctx->opt.precision != HELP_PREC_MIXED)
        return fail(ctx, HELP_E_ARG, "matvec: FP32 copy exists only with HELP_PREC_MIXED");
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    const int nb = spmv_blocks(ctx);
    if (op == HELP_OP_A || op == HELP_OP_AT) {
        if (fp32) return fail(ctx, HELP_E_ARG, "matvec: A / A^T only in FP64");
        const bool t = op == HELP_OP_AT;
        const SpmvView<double> M = t ? view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->avT)
                                     : view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->av);
        CK(spmv_launch<double>(kEpiStore, M, (const double*)x, (double*)y, nullptr, nullptr, nullptr, 0.0, nb,
                               kSpmvThreads, st));
        return HELP_OK;
    }
    if (op == HELP_OP_B || op == HELP_OP_BT) {
        const bool t = op == HELP_OP_BT;
        if (fp32) {
            const SpmvView<float> M = t ? view<float>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT32, true)
                                        : view<float>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv32, true);
            CK(spmv_launch<float>(kEpiStore, M, (const float*)x, (float*)y, nullptr, nullptr, nullptr, 0.0, nb,
                                  kSpmvThreads, st));
        } else {
            const SpmvView<double> M = t ? view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT, true)
                                         : view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv, true);
            CK(spmv_launch<double>(kEpiStore, M, (const double*)x, (double*)y, nullptr, nullptr, nullptr, 0.0, nb,
                                   kSpmvThreads, st));
        }
        return HELP_OK;
    }
    if (op != HELP_OP_ADAT) return fail(ctx, HELP_E_ARG, "matvec: unknown op");
    if (fp32) {
        CK(spmv_launch<float>(kEpiStore, view<float>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT32, true), (const float*)x,
                              ctx->t32.as<float>(), nullptr, nullptr, nullptr, 0.0, nb, kSpmvThreads, st));
        CK(spmv_launch<float>(kEpiAddDelta, view<float>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv32, true), ctx->t32.as<float>(),
                              (float*)y, (const float*)x, nullptr, nullptr, ctx->opt.delta, nb, kSpmvThreads, st));
    } else {
        CK(spmv_launch<double>(kEpiStore, view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->bvT, true), (const double*)x,
                               ctx->t.as<double>(), nullptr, nullptr, nullptr, 0.0, nb, kSpmvThreads, st));
        CK(spmv_launch<double>(kEpiAddDelta, view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->bv, true), ctx->t.as<double>(),
                               (double*)y, (const double*)x, nullptr, nullptr, ctx->opt.delta, nb, kSpmvThreads, st));
    }
    return HELP_OK;
}

int help_pcg_matvec_dev(help_pcg* ctx, int32_t op, int32_t fp32, const void* x, void* y, void* stream) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_matvec_dev_body(ctx, op, fp32, x, y, stream); });
}

static int help_pcg_matvec_body(help_pcg* ctx, int32_t op, const double* x, double* y) {
    if (!ctx || !x || !y) return HELP_E_ARG;
    if (!ctx->constructed) return fail(ctx, HELP_E_ARG, "matvec: construct first");
    CK(cudaSetDevice(ctx->device));
    const size_t nin = (op == HELP_OP_A || op == HELP_OP_B) ? ctx->n : ctx->m;
    const size_t nout = (op == HELP_OP_AT || op == HELP_OP_BT) ? ctx->n : ctx->m;
    if (op < HELP_OP_A || op > HELP_OP_BT) return fail(ctx, HELP_E_ARG, "matvec: unknown op");
    if (op >= HELP_OP_ADAT && !ctx->renewed) return fail(ctx, HELP_E_ARG, "matvec: renew first");
    int rc = h2d_direct(ctx, ctx->xacc.as<double>(), x, nin);
    // with direct host access the last pass stores into y itself where its
    // rows come in index order (A, A^T); the sliced layout's (B, B^T and the
    // second pass of A D^-1 A^T) stores into device memory, and one coalesced
    // copy kernel writes y
    const bool sliced = op != HELP_OP_A && op != HELP_OP_AT;
    void* out = (ctx->host_direct && !sliced) ? (void*)y : ctx->res.p;
    if (!rc) rc = help_pcg_matvec_dev(ctx, op, 0, ctx->xacc.p, out, (void*)ctx->stream);
    if (!rc && ctx->host_direct && sliced) {
        const cudaError_t e = vec_copy(ctx->res.as<double>(), y, (int64_t)nout, ctx->num_sms, ctx->stream);
        if (e != cudaSuccess) rc = fail_cuda(ctx, e, "matvec");
    }
    if (rc || ctx->host_direct) {
        // no kernel may still touch x or y after we return
        const cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (!rc && e != cudaSuccess) rc = fail_cuda(ctx, e, "matvec");
        return rc;
    }
    return d2h(ctx, y, ctx->res.as<double>(), nout);
}

int help_pcg_matvec(help_pcg* ctx, int32_t op, const double* x, double* y) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_matvec_body(ctx, op, x, y); });
}

static int help_pcg_matvec_acc_body(help_pcg* ctx, int32_t transpose, int32_t sign, const double* v, double* dest) {
    if (!ctx || !v || !dest || (sign != 1 && sign != -1)) return HELP_E_ARG;
    if (!ctx->constructed) return fail(ctx, HELP_E_ARG, "matvec: construct first");
    CK(cudaSetDevice(ctx->device));
    const size_t nin = transpose ? ctx->m : ctx->n, nout = transpose ? ctx->n : ctx->m;
    int rc = h2d_direct(ctx, ctx->xacc.as<double>(), v, nin);
    if (!rc) rc = h2d_direct(ctx, ctx->res.as<double>(), dest, nout);
    if (!rc) {
        const SpmvView<double> M = transpose ? view<double>(ctx->pl_csc, ctx->cp, ctx->ri, ctx->avT)
                                             : view<double>(ctx->pl_csr, ctx->rp, ctx->ci, ctx->av);
        // with direct host access the pass stores its rows straight into dest
        // (rows in index order: a warp's stores are contiguous)
        double* out = ctx->host_direct ? dest : ctx->x2.as<double>();
        const cudaError_t e = spmv_launch<double>(kEpiAcc, M, ctx->xacc.as<double>(), out, ctx->res.as<double>(),
                                                  nullptr, nullptr, (double)sign, spmv_blocks(ctx), kSpmvThreads,
                                                  ctx->stream);
        if (e != cudaSuccess) rc = fail(ctx, HELP_E_CUDA, cudaGetErrorString(e));
    }
    if (rc || ctx->host_direct) {
        // no kernel may still touch v or dest after we return
        const cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (!rc && e != cudaSuccess) rc = fail_cuda(ctx, e, "matvec");
        return rc;
    }
    return d2h(ctx, dest, ctx->x2.as<double>(), nout);
}

int help_pcg_matvec_acc(help_pcg* ctx, int32_t transpose, int32_t sign, const double* v, double* dest) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_matvec_acc_body(ctx, transpose, sign, v, dest); });
}

static int help_pcg_precond_apply_body(help_pcg* ctx, const double* r, double* z) {
    if (!ctx || !r || !z) return HELP_E_ARG;
    if (!ctx->renewed) return fail(ctx, HELP_E_ARG, "precond: renew first");
    CK(cudaSetDevice(ctx->device));
    int rc = h2d(ctx, ctx->r0.as<double>(), r, ctx->m);
    if (rc) return rc;
    CK(vec_fill(ctx->xacc.as<double>(), 0.0, ctx->m, ctx->stream));
    CK(vec_fill(ctx->p1.as<double>(), 0.0, ctx->m, ctx->stream));
    CgResult res;
    rc = run_pcg<double>(ctx, ctx->xacc.as<double>(), ctx->r0.as<double>(), 0.0, 1, 1, &res);
    if (rc) return rc;
    return d2h(ctx, z, ctx->p1.as<double>(), ctx->m);
}

int help_pcg_precond_apply(help_pcg* ctx, const double* r, double* z) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_precond_apply_body(ctx, r, z); });
}

static int help_pcg_get_pivots_body(help_pcg* ctx, int32_t* pivots, double* diag_g, double* diag_s) {
    if (!ctx) return HELP_E_ARG;
    if (!ctx->renewed) return fail(ctx, HELP_E_ARG, "pivots: renew first");
    CK(cudaSetDevice(ctx->device));
    if (pivots && ctx->k > 0) {
        CK(cudaMemcpyAsync(pivots, ctx->piv.p, 4 * (size_t)ctx->k, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    int rc = HELP_OK;
    if (diag_g) rc = d2h(ctx, diag_g, ctx->diag.as<double>(), ctx->m);
    if (!rc && diag_s) {
        rc = d2h(ctx, diag_s, ctx->dsinv.as<double>(), ctx->m);
        for (int32_t i = 0; !rc && i < ctx->m; ++i) diag_s[i] = diag_s[i] != 0.0 ? 1.0 / diag_s[i] : 0.0;
    }
    return rc;
}

int help_pcg_get_pivots(help_pcg* ctx, int32_t* pivots, double* diag_g, double* diag_s) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_get_pivots_body(ctx, pivots, diag_g, diag_s); });
}

static int help_pcg_cg_body(help_pcg* ctx, const double* b, double* x, int64_t* iters) {
    if (!ctx || !b || !x) return HELP_E_ARG;
    if (!ctx->renewed) return fail(ctx, HELP_E_ARG, "cg: renew first");
    CK(cudaSetDevice(ctx->device));
    int rc = h2d(ctx, ctx->r0.as<double>(), b, ctx->m);
    if (rc) return rc;
    CK(vec_fill(ctx->x.as<double>(), 0.0, ctx->m, ctx->stream));
    CgResult res;
    ctx->solve_kernel_ms = 0;
    ctx->solve_launches = 0;
    rc = run_pcg<double>(ctx, ctx->x.as<double>(), ctx->r0.as<double>(), ctx->opt.cg_tol, ctx->opt.cg_max_iter, 0, &res);
    if (rc) return rc;
    if (iters) *iters = res.iterations;
    // device time of this CG run, for iteration-rate measurements
    ctx->stats.cg_iterations = res.iterations;
    ctx->stats.cg_kernel_ms = ctx->solve_kernel_ms;
    ctx->stats.cg_launches = ctx->solve_launches;
    return d2h(ctx, x, ctx->x.as<double>(), ctx->m);
}

int help_pcg_cg(help_pcg* ctx, const double* b, double* x, int64_t* iters) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_cg_body(ctx, b, x, iters); });
}

static int help_pcg_cg_f32_body(help_pcg* ctx, const double* b, double* x, int64_t* iters) {
    if (!ctx || !b || !x) return HELP_E_ARG;
    if (!ctx->renewed) return fail(ctx, HELP_E_ARG, "cg_f32: renew first");
    if (ctx->opt.precision != HELP_PREC_MIXED)
        return fail(ctx, HELP_E_ARG, "cg_f32: the context holds no FP32 copies (create it with HELP_PREC_MIXED)");
    CK(cudaSetDevice(ctx->device));
    const int m = ctx->m;
    int rc = h2d(ctx, ctx->r0.as<double>(), b, m);
    if (rc) return rc;
    CK(vec_to_f32(ctx->r0.as<double>(), ctx->r032.as<float>(), m, ctx->stream));
    CK(vec_fill_f32(ctx->x32.as<float>(), 0.0f, m, ctx->stream));
    CgResult res;
    ctx->solve_kernel_ms = 0;
    ctx->solve_launches = 0;
    ctx->solve_iters_f32 = 0;
    rc = run_pcg<float>(ctx, ctx->x32.as<float>(), ctx->r032.as<float>(), ctx->opt.cg_tol, ctx->opt.cg_max_iter, 0, &res);
    if (rc) return rc;
    if (iters) *iters = res.iterations;
    ctx->stats.cg_iterations = res.iterations;
    ctx->stats.cg_iterations_fp32 = res.iterations;
    ctx->stats.cg_kernel_ms = ctx->solve_kernel_ms;
    ctx->stats.cg_launches = ctx->solve_launches;
    CK(vec_fill(ctx->x.as<double>(), 0.0, m, ctx->stream));
    CK(vec_add_f32(ctx->x.as<double>(), ctx->x32.as<float>(), m, ctx->stream));
    return d2h(ctx, x, ctx->x.as<double>(), m);
}

int help_pcg_cg_f32(help_pcg* ctx, const double* b, double* x, int64_t* iters) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_cg_f32_body(ctx, b, x, iters); });
}

static int help_pcg_attach_mlp_body(help_pcg* ctx, help_mlp* mlp) {
    if (!ctx) return HELP_E_ARG;
    if (mlp && help_mlp_device(mlp) != ctx->device)
        return fail(ctx, HELP_E_ARG, "attach_mlp: the model lives on another device");
    if (!mlp && ctx->mlp_active && ctx->renewed) {
        CK(cudaSetDevice(ctx->device));
        int rc = learned_restore(ctx);
        if (rc) return rc;
        CK(cudaStreamSynchronize(ctx->stream));
    }
    ctx->mlp = mlp;
    return HELP_OK;
}

int help_pcg_attach_mlp(help_pcg* ctx, help_mlp* mlp) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_attach_mlp_body(ctx, mlp); });
}

int help_pcg_set_solve_slots(help_pcg* ctx, const int32_t* slots, int32_t n) {
    if (!ctx || n < 0 || n > kSolveSlots || (n > 0 && !slots)) return HELP_E_ARG;
    for (int32_t i = 0; i < n; ++i)
        if (slots[i] < 0 || slots[i] >= kSolveSlots) return HELP_E_ARG;
    for (int32_t i = 0; i < n; ++i) ctx->slot_map[i] = slots[i];
    ctx->slot_map_n = n;
    return HELP_OK;
}

static int help_pcg_share_solution_body(help_pcg* dst, int32_t dst_slot, help_pcg* src, int32_t src_slot) {
    if (!dst || !src || dst_slot < 0 || dst_slot >= kSolveSlots || src_slot < 0 || src_slot >= kSolveSlots)
        return HELP_E_ARG;
    if (!dst->constructed || !src->constructed || dst->m != src->m || dst->device != src->device)
        return fail(dst, HELP_E_ARG, "share_solution: both contexts constructed with the same matrix, same device");
    help_pcg* ctx = dst;  // CK reports on the destination
    const bool have = src->mlp && src->x2_have[src->x2_cur][src_slot];
    dst->x2_have[dst->x2_cur][dst_slot] = false;
    if (!have || !dst->mlp) return HELP_OK;
    CK(cudaSetDevice(dst->device));
    CK(cudaStreamSynchronize(src->stream));  // src's copy of that solution is complete
    CK(dst->x2h[dst->x2_cur][dst_slot].ensure(8 * (size_t)dst->m));
    CK(cudaMemcpyAsync(dst->x2h[dst->x2_cur][dst_slot].p, src->x2h[src->x2_cur][src_slot].p, 8 * (size_t)dst->m,
                       cudaMemcpyDeviceToDevice, dst->stream));
    CK(cudaStreamSynchronize(dst->stream));
    dst->x2_have[dst->x2_cur][dst_slot] = true;
    return HELP_OK;
}

int help_pcg_share_solution(help_pcg* dst, int32_t dst_slot, help_pcg* src, int32_t src_slot) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_share_solution_body(dst, dst_slot, src, src_slot); });
}

static int help_pcg_features_body(help_pcg* ctx, int32_t slot, float* x) {
    if (!ctx || !x || slot < 0 || slot >= kSolveSlots) return HELP_E_ARG;
    if (!ctx->renewed) return fail(ctx, HELP_E_ARG, "features: renew first");
    CK(cudaSetDevice(ctx->device));
    int rc = learned_features(ctx, slot, nullptr, x);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return HELP_OK;
}

int help_pcg_features(help_pcg* ctx, int32_t slot, float* x) {
    return c_guard(HELP_E_NOMEM, [&] { return help_pcg_features_body(ctx, slot, x); });
}

static int help_adat_assemble_body(help_pcg* ctx, const double* w, int32_t* row_ptr, int32_t* col, double* val, int64_t* nnz) {
    if (!ctx || !w || !row_ptr || !nnz) return HELP_E_ARG;
    if (!ctx->constructed) return fail(ctx, HELP_E_ARG, "adat: construct first");
    CK(cudaSetDevice(ctx->device));
    const int m = ctx->m;
    int rc = h2d(ctx, ctx->res.as<double>(), w, ctx->n);
    if (rc) return rc;
    int* cnt = ctx->cr_cnt.as<int>();
    CK(adat_count(ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->cp.as<int>(), ctx->ri.as<int>(), m, cnt, ctx->stream));
    std::vector<int32_t> hc((size_t)m);
    CK(cudaMemcpyAsync(hc.data(), cnt, 4 * (size_t)m, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    // rows whose contributions overflow the per-warp sort: the heavy-row kernel
    std::vector<int32_t> heavy;
    for (int i = 0; i < m; ++i)
        if (hc[i] < 0) heavy.push_back(i);
    const int nh = (int)heavy.size();
    int* d_heavy = nullptr;
    int* d_hcnt = nullptr;
    double* h_acc = nullptr;
    int* h_stamp = nullptr;
    unsigned* h_bits = nullptr;
    size_t R = 0;
    int slots = 0;
    if (nh > 0) {
        CK(ctx->adat_heavy_list.ensure(8 * (size_t)nh + 16));
        d_heavy = ctx->adat_heavy_list.as<int>();
        d_hcnt = d_heavy + nh + (nh & 1);
        CK(cudaMemcpyAsync(d_heavy, heavy.data(), 4 * (size_t)nh, cudaMemcpyHostToDevice, ctx->stream));
        CK(adat_heavy_range(d_heavy, nh, ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->cp.as<int>(), ctx->ri.as<int>(),
                            d_hcnt, ctx->stream));
        std::vector<int32_t> hr((size_t)nh);
        CK(cudaMemcpyAsync(hr.data(), d_hcnt, 4 * (size_t)nh, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        for (int h = 0; h < nh; ++h) R = std::max(R, (size_t)hr[h]);
        // one accumulator slot per warp: at most 2 warps per SM, and at most
        // ~1 GiB of slots (acc + stamp + bitmap = 12.125 bytes per entry)
        const size_t per_slot = 12 * R + 4 * ((R + 31) / 32) + 64;
        size_t cap = ((size_t)1 << 30) / per_slot;
        slots = (int)std::min<size_t>(std::min<size_t>((size_t)nh, (size_t)2 * ctx->num_sms), std::max<size_t>(cap, 1));
        slots = (slots + 3) & ~3;
        CK(ctx->adat_heavy_slots.ensure(per_slot * (size_t)slots + 256));
        h_acc = ctx->adat_heavy_slots.as<double>();
        h_stamp = reinterpret_cast<int*>(h_acc + (size_t)slots * R);
        h_bits = reinterpret_cast<unsigned*>(h_stamp + (size_t)slots * R);
        CK(cudaMemsetAsync(h_stamp, 0xFF, 4 * (size_t)slots * R, ctx->stream));
        CK(cudaMemsetAsync(h_bits, 0, 4 * (size_t)slots * ((R + 31) / 32), ctx->stream));
        CK(adat_heavy(d_heavy, nh, ctx->rp.as<int>(), ctx->ci.as<int>(), nullptr, ctx->cp.as<int>(),
                      ctx->ri.as<int>(), nullptr, nullptr, h_acc, h_stamp, h_bits, R, slots, d_hcnt, nullptr, nullptr,
                      nullptr, ctx->stream));
        std::vector<int32_t> hh((size_t)nh);
        CK(cudaMemcpyAsync(hh.data(), d_hcnt, 4 * (size_t)nh, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        for (int h = 0; h < nh; ++h) hc[heavy[h]] = hh[h];
    }
    int64_t total = 0;
    row_ptr[0] = 0;
    for (int i = 0; i < m; ++i) {
        total += hc[i];
        if (total > 2147483647LL) return fail(ctx, HELP_E_ARG, "adat: result exceeds int32 indexing");
        row_ptr[i + 1] = (int32_t)total;
    }
    *nnz = total;
    if (!col || !val) return HELP_OK;
    CK(ctx->adat_tmp.ensure(4 * ((size_t)m + 1) + 12 * (size_t)std::max<int64_t>(total, 1) + 16));
    int* drp = ctx->adat_tmp.as<int>();
    int* dci = drp + m + 1 + ((m + 1) & 1);
    double* dv = reinterpret_cast<double*>(dci + total + (total & 1));
    CK(cudaMemcpyAsync(drp, row_ptr, 4 * ((size_t)m + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(adat_fill(ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->av.as<double>(), ctx->cp.as<int>(), ctx->ri.as<int>(),
                 ctx->avT.as<double>(), ctx->res.as<double>(), m, drp, dci, dv, ctx->stream));
    if (nh > 0) {
        CK(cudaMemsetAsync(h_stamp, 0xFF, 4 * (size_t)slots * R, ctx->stream));
        CK(adat_heavy(d_heavy, nh, ctx->rp.as<int>(), ctx->ci.as<int>(), ctx->av.as<double>(), ctx->cp.as<int>(),
                      ctx->ri.as<int>(), ctx->avT.as<double>(), ctx->res.as<double>(), h_acc, h_stamp, h_bits, R, slots,
                      d_hcnt, drp, dci, dv, ctx->stream));
    }
    CK(cudaMemcpyAsync(col, dci, 4 * (size_t)total, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(val, dv, 8 * (size_t)total, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HELP_OK;
}

int help_adat_assemble(help_pcg* ctx, const double* w, int32_t* row_ptr, int32_t* col, double* val, int64_t* nnz) {
    return c_guard(HELP_E_NOMEM, [&] { return help_adat_assemble_body(ctx, w, row_ptr, col, val, nnz); });
}

}  // extern "C"
