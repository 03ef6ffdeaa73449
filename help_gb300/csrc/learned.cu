// Solver side of the learned part: per-row features of the normal equations
// (input of the MLP in mlp.cu), and the two uses of its output -- a
// correction of the Schur diagonal of the partial-Cholesky preconditioner
// and a per-row scale of the warm start.
#include <cuda_bf16.h>

#include "common.cuh"
#include "mlp.h"

namespace help {
namespace {

constexpr float kDiagClamp = 2.0f;  // |log-factor| of the D_S correction
constexpr int kFeatures = 11;       // features in use; the rest of the row is zero

// Writes the normalised BF16 row of X, or (X null) the raw FP32 row of R.
__global__ void __launch_bounds__(256) k_features(const int* __restrict__ rp, const int* __restrict__ ci,
                                                  const double* __restrict__ d, const double* __restrict__ diag,
                                                  const double* __restrict__ dsinv, const int* __restrict__ pivpos,
                                                  const double* __restrict__ xprev, const double* xprev_sumsq,
                                                  const double* __restrict__ dprev, int m,
                                                  const MlpDevWeights* __restrict__ w, __nv_bfloat16* __restrict__ X,
                                                  float* __restrict__ R) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int b = rp[i], e = rp[i + 1];
    float s = 0.f, s2 = 0.f, lo = 0.f, hi = 0.f, dm = 0.f, dx = 0.f;
    for (int q = b; q < e; ++q) {
        const int j = ci[q];
        const float l = log10f((float)d[j]);
        s += l;
        s2 += l * l;
        lo = (q == b) ? l : fminf(lo, l);
        hi = (q == b) ? l : fmaxf(hi, l);
        if (dprev) {
            const float c = l - log10f((float)dprev[j]);
            dm += c;
            dx = fmaxf(dx, fabsf(c));
        }
    }
    const int len = e - b;
    const float mean = len > 0 ? s / len : 0.f;
    const float var = len > 0 ? fmaxf(s2 / len - mean * mean, 0.f) : 0.f;
    const double dg = diag[i];
    float f[HELP_MLP_IN];
    f[0] = dg > 0.0 ? log10f((float)dg) : -30.f;
    f[1] = mean;
    f[2] = sqrtf(var);
    f[3] = lo;
    f[4] = hi;
    f[5] = log2f(1.f + (float)len);
    const bool piv = pivpos[i] >= 0;
    const double ratio = (!piv && dsinv[i] > 0.0 && dg > 0.0) ? 1.0 / (dsinv[i] * dg) : 1.0;
    f[6] = piv ? 0.f : log10f((float)ratio);
    f[7] = piv ? 1.f : 0.f;
    float xf = 0.f;
    if (xprev) {
        const double ss = *xprev_sumsq;
        if (ss > 0.0) xf = (float)(xprev[i] / sqrt(ss / m));
    }
    f[8] = xf;
    f[9] = len > 0 ? dm / len : 0.f;  // mean change of log10 d since the previous renew
    f[10] = dx;                        // largest change
#pragma unroll
    for (int k = kFeatures; k < HELP_MLP_IN; ++k) f[k] = 0.f;
    if (!X) {
#pragma unroll
        for (int k = 0; k < HELP_MLP_IN; ++k) R[(size_t)i * HELP_MLP_IN + k] = f[k];
        return;
    }
    uint32_t* out = reinterpret_cast<uint32_t*>(X + (size_t)i * HELP_MLP_IN);
#pragma unroll
    for (int k = 0; k < HELP_MLP_IN; k += 2) {
        const float a = k < kFeatures ? (f[k] - w->mean[k]) * w->scale[k] : 0.f;
        const float c = k + 1 < kFeatures ? (f[k + 1] - w->mean[k + 1]) * w->scale[k + 1] : 0.f;
        const __nv_bfloat162 v = __floats2bfloat162_rn(a, c);
        out[k / 2] = *reinterpret_cast<const uint32_t*>(&v);
    }
}

__global__ void __launch_bounds__(256) k_apply_diag(const float* __restrict__ out, const int* __restrict__ pivpos,
                                                    double* __restrict__ dsinv, float* __restrict__ dsinv32, int m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || pivpos[i] >= 0) return;
    const float o = fminf(fmaxf(out[2 * (size_t)i], -kDiagClamp), kDiagClamp);
    const double v = dsinv[i] * (double)expf(-o);
    dsinv[i] = v;
    if (dsinv32) dsinv32[i] = (float)v;
}

__global__ void __launch_bounds__(256) k_warm_vector(const float* __restrict__ out, const double* __restrict__ xprev,
                                                     double* __restrict__ v, int m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) v[i] = (double)out[2 * (size_t)i + 1] * xprev[i];
}

}  // namespace

cudaError_t mlp_features(const int* rp, const int* ci, const double* d, const double* diag, const double* dsinv,
                         const int* pivpos, const double* xprev, const double* xprev_sumsq, const double* dprev,
                         int m, const MlpDevWeights* w, __nv_bfloat16* X, float* R, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_features<<<(m + 255) / 256, 256, 0, st>>>(rp, ci, d, diag, dsinv, pivpos, xprev, xprev_sumsq, dprev, m, w, X, R);
    return cudaGetLastError();
}

cudaError_t mlp_apply_diag(const float* out, const int* pivpos, double* dsinv, float* dsinv32, int m,
                           cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_apply_diag<<<(m + 255) / 256, 256, 0, st>>>(out, pivpos, dsinv, dsinv32, m);
    return cudaGetLastError();
}

cudaError_t mlp_warm_vector(const float* out, const double* xprev, double* v, int m, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_warm_vector<<<(m + 255) / 256, 256, 0, st>>>(out, xprev, v, m);
    return cudaGetLastError();
}

}  // namespace help
