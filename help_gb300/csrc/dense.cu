// Dense k x k pivot block: W = G11^-1 by FP64 Cholesky G11 = L L^T,
// X = L^-1 and W = X^T X.
//
// The reference factors its pivot block as a unit-lower LDL^T by left-looking
// column updates (PCG.cpp:80-97) and inverts L11 by elimination
// (PCG.cpp:119-133); the inverse is then applied as an explicit matrix
// (PCG.cpp:135-195).  Here the same operator G11^-1 is formed once per renew
// with blocked kernels (32 x 32 diagonal blocks in shared memory, tiled panel
// and trailing updates), in FP64 as the precision policy requires.  tcgen05
// has no FP64 kind and GB300's FP64 rate is the same on the legacy DMMA path
// as on the FP64 pipes, so these are plain FP64 FMA kernels.
//
// A pivot that falls below 1e-14 of its original diagonal (a numerically
// singular pivot block) is raised to that floor and counted.
#include "common.cuh"
#include "kernels.h"

namespace help {

namespace {

constexpr int NB = 32;

// Factor the kb x kb diagonal block at (j0, j0) in place (lower) and write its
// inverse into linv (NB x NB, row-major).  1024 threads: (r, c) = (ty, tx).
__global__ void k_potrf_diag(double* __restrict__ A, int k, int j0, int kb, double* __restrict__ linv,
                             const double* __restrict__ orig_diag, int* __restrict__ regularised) {
    __shared__ double L[NB][NB + 1];
    __shared__ double X[NB][NB + 1];
    __shared__ double fl[NB], rdiag[NB];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    L[ty][tx] = (ty < kb && tx < kb && tx <= ty) ? A[(size_t)(j0 + ty) * k + j0 + tx] : 0.0;
    X[ty][tx] = 0.0;
    if (ty == 0) fl[tx] = tx < kb ? fmax(1.0e-14 * orig_diag[j0 + tx], 1.0e-300) : 1.0;
    __syncthreads();
    for (int c = 0; c < kb; ++c) {
        if (threadIdx.x == 0) {
            double piv = L[c][c];
            if (!(piv > fl[c])) {
                piv = fl[c];
                atomicAdd(regularised, 1);
            }
            const double sq = sqrt(piv);
            L[c][c] = sq;
            rdiag[c] = 1.0 / sq;
        }
        __syncthreads();
        if (tx == 0 && ty > c && ty < kb) L[ty][c] *= rdiag[c];
        __syncthreads();
        if (ty > c && ty < kb && tx > c && tx <= ty) L[ty][tx] = fma(-L[ty][c], L[tx][c], L[ty][tx]);
        __syncthreads();
    }
    // inverse of the lower-triangular block by rows: X[r][c] for every column
    // c < r at once (thread tx = c), using the rows above it
    if (ty == 0 && tx < kb) X[tx][tx] = rdiag[tx];
    __syncthreads();
    for (int r = 1; r < kb; ++r) {
        if (ty == 0 && tx < r) {
            double s = 0.0;
            for (int l = tx; l < r; ++l) s = fma(L[r][l], X[l][tx], s);
            X[r][tx] = -s * rdiag[r];
        }
        __syncthreads();
    }
    if (ty < kb && tx < kb && tx <= ty) A[(size_t)(j0 + ty) * k + j0 + tx] = L[ty][tx];
    linv[ty * NB + tx] = (ty < kb && tx < kb) ? X[ty][tx] : 0.0;
}

// Panel below the diagonal block: L[i, j0:j0+kb] = A[i, j0:j0+kb] * Linv^T for
// rows i in [j0 + kb, k).  Block: 32 rows x 32 columns.
__global__ void k_trsm_panel(double* __restrict__ A, int k, int j0, int kb, const double* __restrict__ linv) {
    __shared__ double R[NB][NB + 1];
    __shared__ double Li[NB][NB + 1];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = j0 + kb + blockIdx.x * NB + ty;
    R[ty][tx] = (i < k && tx < kb) ? A[(size_t)i * k + j0 + tx] : 0.0;
    Li[ty][tx] = linv[ty * NB + tx];
    __syncthreads();
    if (i < k && tx < kb) {
        double s = 0.0;
        for (int l = 0; l <= tx; ++l) s = fma(R[ty][l], Li[tx][l], s);
        A[(size_t)i * k + j0 + tx] = s;
    }
}

// Trailing update of the lower triangle: A[i][l] -= sum_c P[i][c] P[l][c] for
// i, l >= s0, l <= i, with P = A[:, j0:j0+kb].  64 x 64 tiles, 256 threads.
__global__ void k_syrk_lower(double* __restrict__ A, int k, int j0, int kb, int s0) {
    const int tile_i = blockIdx.y, tile_l = blockIdx.x;
    if (tile_l > tile_i) return;
    __shared__ double Pi[64][NB + 1];
    __shared__ double Pl[64][NB + 1];
    const int i0 = s0 + tile_i * 64, l0 = s0 + tile_l * 64;
    for (int t = threadIdx.x; t < 64 * NB; t += blockDim.x) {
        const int r = t / NB, c = t % NB;
        Pi[r][c] = (i0 + r < k && c < kb) ? A[(size_t)(i0 + r) * k + j0 + c] : 0.0;
        Pl[r][c] = (l0 + r < k && c < kb) ? A[(size_t)(l0 + r) * k + j0 + c] : 0.0;
    }
    __syncthreads();
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;  // 16 x 16 threads, 4 x 4 outputs each
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int c = 0; c < kb; ++c) {
        double vi[4], vl[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) vi[a] = Pi[tr + 16 * a][c];
#pragma unroll
        for (int b = 0; b < 4; ++b) vl[b] = Pl[tc + 16 * b][c];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = fma(vi[a], vl[b], acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = i0 + tr + 16 * a, l = l0 + tc + 16 * b;
            if (i < k && l < k && l <= i) A[(size_t)i * k + l] -= acc[a][b];
        }
}

// Triangular inverse X = L^-1 by recursive halving, level by level: with
// L = [L_A 0; B L_C] on a node of 2 n rows, X = [X_A 0; -X_C B X_A X_C].
// Level n = 32, 64, ... doubles the nodes' size; each level is two batched
// GEMM launches over all its nodes (T = B X_A, then X_21 = -X_C T), so the
// inverse takes 2 log2(nblk) launches instead of nblk dependent steps.  X
// has the padded order kp = 32 * 2^ceil(log2 nblk); rows and columns past k
// are an identity block that couples to nothing.  The zeros above the
// diagonal of X_A and X_C are skipped a K-slab at a time.
constexpr int TG = 64;   // output tile
constexpr int TK = 16;   // K slab

// mode 0: T = B X_A   (A operand = L rows o+n.., cols o..; B operand = X_A)
// mode 1: X21 = -X_C T (A operand = X_C; B operand = T)
template <int MODE>
__global__ void __launch_bounds__(256) k_trtri_level(const double* __restrict__ L, int k, double* __restrict__ X,
                                                     int kp, double* __restrict__ T, int n) {
    const int node = blockIdx.z;
    const int o = node * 2 * n;
    if (o + n >= k) return;  // B is entirely past k: this node's X_21 stays zero
    const int i0 = blockIdx.y * TG, j0 = blockIdx.x * TG;
    if (i0 >= n || j0 >= n) return;
    double* Tn = T + (size_t)node * n * n;
    __shared__ double As[TG][TK + 1];
    __shared__ double Bs[TK][TG + 1];
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    // K range: mode 0 skips l < j0 (X_A lower), mode 1 skips l > i0 + TG - 1 (X_C lower)
    const int kbeg = MODE == 0 ? (j0 / TK) * TK : 0;
    const int kend = MODE == 0 ? n : min(n, i0 + TG);
    for (int l0 = kbeg; l0 < kend; l0 += TK) {
        for (int t = threadIdx.x; t < TG * TK; t += blockDim.x) {
            const int r = t / TK, c = t % TK;
            const int gi = i0 + r, gl = l0 + c;
            double v = 0.0;
            if (gi < n && gl < n) {
                if (MODE == 0) {
                    const int row = o + n + gi, col = o + gl;
                    v = (row < k && col < k) ? L[(size_t)row * k + col] : 0.0;
                } else {
                    v = X[(size_t)(o + n + gi) * kp + (o + n + gl)];
                }
            }
            As[r][c] = v;
        }
        for (int t = threadIdx.x; t < TK * TG; t += blockDim.x) {
            const int r = t / TG, c = t % TG;
            const int gl = l0 + r, gj = j0 + c;
            double v = 0.0;
            if (gl < n && gj < n) v = MODE == 0 ? X[(size_t)(o + gl) * kp + (o + gj)] : Tn[(size_t)gl * n + gj];
            Bs[r][c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < TK; ++c) {
            double va[4], vb[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) va[a] = As[tr + 16 * a][c];
#pragma unroll
            for (int b = 0; b < 4; ++b) vb[b] = Bs[c][tc + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fma(va[a], vb[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gi = i0 + tr + 16 * a, gj = j0 + tc + 16 * b;
            if (gi < n && gj < n) {
                if (MODE == 0) Tn[(size_t)gi * n + gj] = acc[a][b];
                else X[(size_t)(o + n + gi) * kp + (o + gj)] = -acc[a][b];
            }
        }
}

// Diagonal blocks of X: the 32 x 32 inverses, identity past k.
__global__ void k_place_linv(double* __restrict__ X, int kp, int nblk, const double* __restrict__ linv_all) {
    const int b = blockIdx.x;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const double v = b < nblk ? linv_all[(size_t)b * NB * NB + ty * NB + tx] : (tx == ty ? 1.0 : 0.0);
    X[(size_t)(b * NB + ty) * kp + b * NB + tx] = v;
}

// W = X^T X for lower-triangular X: W[a][b] = sum_{l >= max(a,b)} X[l][a] X[l][b],
// lower tiles computed, both triangles written.
__global__ void k_xtx(const double* __restrict__ X, int ldx, double* __restrict__ W, int k) {
    const int ta = blockIdx.y, tb = blockIdx.x;
    if (tb > ta) return;
    __shared__ double Xa[16][64 + 1];
    __shared__ double Xb[16][64 + 1];
    const int a0 = ta * 64, b0 = tb * 64;
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    double acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = 0.0;
    for (int l0 = a0; l0 < k; l0 += 16) {  // rows l < a0 contribute nothing to column block a
        for (int t = threadIdx.x; t < 16 * 64; t += blockDim.x) {
            const int r = t / 64, c = t % 64;
            const int l = l0 + r;
            Xa[r][c] = (l < k && a0 + c < k) ? X[(size_t)l * ldx + a0 + c] : 0.0;
            Xb[r][c] = (l < k && b0 + c < k) ? X[(size_t)l * ldx + b0 + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            double va[4], vb[4];
#pragma unroll
            for (int p = 0; p < 4; ++p) va[p] = Xa[r][tr + 16 * p];
#pragma unroll
            for (int q = 0; q < 4; ++q) vb[q] = Xb[r][tc + 16 * q];
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = fma(va[p], vb[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int a = a0 + tr + 16 * p, b = b0 + tc + 16 * q;
            if (a < k && b < k && b <= a) {
                W[(size_t)a * k + b] = acc[p][q];
                W[(size_t)b * k + a] = acc[p][q];
            }
        }
}

__global__ void k_copy_diag(const double* __restrict__ A, int k, double* __restrict__ dg) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) dg[i] = A[(size_t)i * k + i];
}

}  // namespace

// padded order of X: 32 * (smallest power of two >= the block count)
int padded_order(int k) {
    const int nblk = (k + NB - 1) / NB;
    int p = 1;
    while (p < nblk) p *= 2;
    return p * NB;
}

size_t dense_work_elems(int k) {
    const size_t nblk = (size_t)(k + NB - 1) / NB;
    const size_t kp = (size_t)padded_order(k);
    return kp * kp + kp * kp / 4 + nblk * NB * NB + (size_t)k + 64;
}

cudaError_t dense_spd_inverse(double* g11, double* W, double* work, int k, int* regularised, cudaStream_t st) {
    if (k <= 0) return cudaSuccess;
    const int nblk = (k + NB - 1) / NB;
    const int kp = padded_order(k);
    double* X = work;                                        // kp * kp
    double* T = X + (size_t)kp * kp;                          // kp * kp / 4 (level temporaries)
    double* linv_all = T + (size_t)kp * kp / 4;               // nblk * NB * NB
    double* orig_diag = linv_all + (size_t)nblk * NB * NB;    // k
    k_copy_diag<<<(k + 255) / 256, 256, 0, st>>>(g11, k, orig_diag);
    for (int jb = 0; jb < nblk; ++jb) {
        const int j0 = jb * NB, kb = (k - j0 < NB) ? k - j0 : NB;
        k_potrf_diag<<<1, NB * NB, 0, st>>>(g11, k, j0, kb, linv_all + (size_t)jb * NB * NB, orig_diag, regularised);
        const int rest = k - j0 - kb;
        if (rest > 0) {
            k_trsm_panel<<<(rest + NB - 1) / NB, NB * NB, 0, st>>>(g11, k, j0, kb, linv_all + (size_t)jb * NB * NB);
            const int tiles = (rest + 63) / 64;
            k_syrk_lower<<<dim3(tiles, tiles), 256, 0, st>>>(g11, k, j0, kb, j0 + kb);
        }
    }
    cudaError_t e = cudaMemsetAsync(X, 0, sizeof(double) * (size_t)kp * kp, st);
    if (e != cudaSuccess) return e;
    k_place_linv<<<kp / NB, NB * NB, 0, st>>>(X, kp, nblk, linv_all);
    for (int n = NB; n < kp; n *= 2) {
        const int tiles = (n + TG - 1) / TG, nodes = kp / (2 * n);
        const dim3 grid(tiles, tiles, nodes);
        k_trtri_level<0><<<grid, 256, 0, st>>>(g11, k, X, kp, T, n);
        k_trtri_level<1><<<grid, 256, 0, st>>>(g11, k, X, kp, T, n);
    }
    const int tiles = (k + 63) / 64;
    k_xtx<<<dim3(tiles, tiles), 256, 0, st>>>(X, kp, W, k);
    return cudaGetLastError();
}

}  // namespace help
