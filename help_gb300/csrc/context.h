// Host-side state of one help_pcg context (one matrix resident on one GPU).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/help_gpu.h"
#include "items.h"
#include "kernels.h"

namespace help {

// Growable device buffer (contents not preserved on growth).
struct DevMem {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b == 0) b = 16;
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// A planned CSR matrix: the split of its rows for spmv_rows (spmv.cuh), one
// per precision (the group-size floor differs).
struct RowSplit {
    DevMem med, lng;
    DevMem seg, lnseg, lbase, tickets, parts;  // segments of long rows (items.h)
    DevMem sorder;                             // short rows in processing order (when uneven)
    int32_t G = 1, short_max = 32, n_med = 0, n_long = 0, n_seg = 0, n_short = 0;
    // sliced layout of the short rows (items.h, SellHost), for B = A D^-1/2:
    // its values (this split's precision) are refreshed from B at each renew
    DevMem sell_ptr, sell_perm, sell_idx, sell_map, sell_val;
    int32_t n_sell = 0, sell_W = 1;
    int64_t sell_entries = 0;
};
struct RowPlan {
    int32_t rows = 0;
    RowSplit s64, s32;
};

// Lanes per short row (spmv.cuh): at least kGmin*, grown until each lane has
// at most kPerLane* nonzeros of an average row.  Measured on GB300 (config 1,
// 2 and 4 passes): FP32 is fastest at ~4 per lane down to groups of 2 (the
// FP32 pass over 6-nonzero rows 74 -> 45 us against a floor of 8 lanes);
// FP64 at 7 per lane: rows of 13 want 2 lanes (4 lanes cost 40 %), rows of
// 21 want 4 (8 lanes cost 13 %), rows of 32 want 8 (28.7 -> 26.6 us).
constexpr int kGminF64 = 2;
constexpr int kPerLaneF64 = 7;
constexpr int kGminF32 = 2;
constexpr int kPerLaneF32 = 4;
// C = G[N, P] gathers a, a k-vector that sits in shared memory or L1, so its
// pass is bound by the FP64 pipe rather than by L2 requests: more nonzeros
// per lane, fewer shuffle adds and idle lanes per row (config 4's C: rows of
// ~85 entries, 16 -> 4 lanes each).
constexpr int kPerLaneCF64 = 24;
constexpr int kPerLaneCF32 = 16;

constexpr int kTopkBins = 256;
constexpr int kGraphIters = 8;    // CG iterations per graph launch
constexpr int kSolveSlots = 4;    // solves per renew whose solutions seed the next renew's
// auto path: single-cluster CG at or below this work per iteration (measured:
// faster than the graph on config 0 (77k), slower from ~250k on)
constexpr int64_t kClusterWorkMax = 150000;

}  // namespace help

struct help_pcg {
    help_pcg_options opt;
    int device = 0;
    int num_sms = 0;
    bool host_direct = false;  // kernels may access pageable host memory (Grace: host page tables)
    cudaStream_t stream = nullptr;
    std::string err;

    // matrix
    int32_t m = 0, n = 0;
    int64_t nnz = 0;
    bool constructed = false;
    bool renewed = false;
    std::vector<int32_t> h_rp, h_cp;  // host copies of the pointers (planning)
    help::DevMem rp, ci, av;          // CSR(A), original values
    help::DevMem cp, ri, avT;         // CSR(A^T) = CSC(A), original values
    help::DevMem bv, bvT;             // B = A D^-1/2 (FP64)
    help::DevMem bv32, bvT32;         // B in FP32 (mixed precision)
    help::RowPlan pl_csr, pl_csc;     // row splits of A and A^T

    // renew state
    int32_t k = 0;
    int64_t nnz_c = 0;
    help::DevMem d, s, diag, dsinv, dsinv32, piv, pivpos;
    help::DevMem keys, hist, flags, scan_tmp;
    help::DevMem bp_ptr, bp_c, bp_v;      // per column of A: pivot entries (c, B value)
    help::DevMem cr_cnt;                  // per row: entries of G[i,P]
    help::DevMem c_rp, c_ci, c_v, c_v32;  // C = G[non-pivot rows, P], CSR over all m rows
    help::DevMem ct_rp, ct_ci, ct_v, ct_v32, ct_blk;  // C^T, CSR over k rows
    help::RowPlan pl_c, pl_ct;
    help::DevMem g11, W, lwork;           // pivot block, its inverse, factor workspace
    std::vector<int32_t> h_tmp;
    int32_t dense_regularised = 0;

    // vectors
    help::DevMem x, r0, r1, z, p0, p1, q, t, a, w;         // FP64 CG
    help::DevMem x32, r032, r132, z32, p032, p132, q32, t32;  // FP32 CG
    help::DevMem u, rhs, b1, b2, x1, x2, res, xacc;         // solve-level FP64 vectors
    help::DevMem partials;
    help::DevMem ctrl;
    help::DevMem adat_tmp;
    help::DevMem adat_heavy_list, adat_heavy_slots;  // heavy rows of the assembly and their accumulators


    const double* last_d = nullptr;
    bool have_prev_x2 = false;
    bool fp32_stagnated = false;      // mixed: FP32 refinement stalled once; FP64 from then on
    double d_spread = 1.0;            // max(d) / min(d) of the last renew

    // learned part (mlp_api.cu): attached model, its per-renew inputs and
    // outputs, the uncorrected D_S^-1, and the solutions of the solve slots
    // of the current and the previous renew
    help_mlp* mlp = nullptr;
    bool mlp_active = false;          // correction applied in this renew (cleared by a fallback)
    help::DevMem mlp_x, mlp_out, dsinv_plain, d_prev;
    bool have_dprev = false;          // d_prev holds the previous renew's d
    help::DevMem x2h[2][help::kSolveSlots];
    bool x2_have[2][help::kSolveSlots] = {};
    int x2_cur = 0;
    int solve_slot = 0;
    // slot of the i-th solve after a renew (help_pcg_set_solve_slots); past
    // slot_map_n, solve i takes slot min(i, kSolveSlots - 1)
    int32_t slot_map[help::kSolveSlots] = {};
    int32_t slot_map_n = 0;
    help_pcg_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // CG graphs (one per precision), re-captured when their arguments change
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    std::vector<unsigned char> graph_args[2];
    int cg_blocks = 0;
    int cluster_cs[2] = {0, 0};       // single-cluster CG: CTAs per cluster (0 = unavailable)
    int resident_cs[2] = {0, 0};      // shared-memory-resident CG (set at renew): CTAs per cluster, 0 = no fit
    help::ResLayout resident_layout[2] = {};
    help::DevMem cg_part;  // 4 x cg_blocks doubles
    help::CgScalars* h_sc = nullptr;  // pinned mirror of the device scalars
    double solve_kernel_ms = 0;       // accumulators for the current solve
    long long solve_iters_f32 = 0;
    int solve_launches = 0;
};
