// Device layout and launchers of the learned part (mlp.cu, learned.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/help_gpu.h"

namespace help {

// Trainable parameters: every offset below HELP_MLP_OFF_MEAN.
constexpr int kMlpGradParams = HELP_MLP_OFF_MEAN;
constexpr int kMlpLossBlocks = 256;

// Weights as the kernels read them (one device struct per model).
struct MlpDevWeights {
    __nv_bfloat16 w1[HELP_MLP_HIDDEN * HELP_MLP_IN];
    __nv_bfloat16 w2[HELP_MLP_HIDDEN * HELP_MLP_HIDDEN];
    __nv_bfloat16 w3[8 * HELP_MLP_HIDDEN];  // rows >= HELP_MLP_OUT stay zero
    float b1[HELP_MLP_HIDDEN];
    float b2[HELP_MLP_HIDDEN];
    float b3[8];                            // entries >= HELP_MLP_OUT stay zero
    float mean[HELP_MLP_IN];                // feature normalisation: (f - mean) * scale
    float scale[HELP_MLP_IN];
};

// Parameter j (trainable layout of help_gpu.h) into the device weights.
__device__ __forceinline__ void mlp_store_param(MlpDevWeights* w, int j, float v) {
    if (j < HELP_MLP_OFF_B1) w->w1[j] = __float2bfloat16(v);
    else if (j < HELP_MLP_OFF_W2) w->b1[j - HELP_MLP_OFF_B1] = v;
    else if (j < HELP_MLP_OFF_B2) w->w2[j - HELP_MLP_OFF_W2] = __float2bfloat16(v);
    else if (j < HELP_MLP_OFF_W3) w->b2[j - HELP_MLP_OFF_B2] = v;
    else if (j < HELP_MLP_OFF_B3) w->w3[j - HELP_MLP_OFF_W3] = __float2bfloat16(v);
    else if (j < HELP_MLP_OFF_MEAN) w->b3[j - HELP_MLP_OFF_B3] = v;
}

int mlp_blocks(long long rows, int num_sms);
cudaError_t mlp_configure();
// out[rows x 2]; H1 / H2 (rows x 64, BF16) kept when not null (training)
cudaError_t mlp_forward(const __nv_bfloat16* X, long long rows, const MlpDevWeights* w, float* out,
                        __nv_bfloat16* H1, __nv_bfloat16* H2, int num_sms, cudaStream_t st);
// Weighted squared error of out against tg (weights wt, all rows x 2):
// loss partials in lpart[0, kMlpLossBlocks), G3 = dL/dout, gradient of the
// trainable parameters into grad (gpart: mlp_blocks(rows) x kMlpGradParams).
cudaError_t mlp_loss_grad(const __nv_bfloat16* X, long long rows, const MlpDevWeights* w, const float* out,
                          const float* tg, const float* wt, float* G3, const __nv_bfloat16* H1,
                          const __nv_bfloat16* H2, double* lpart, float* gpart, float* grad, int num_sms,
                          cudaStream_t st);
cudaError_t mlp_adam(float* prm, float* m1, float* m2, const float* grad, float lr, int step, MlpDevWeights* w,
                     cudaStream_t st);
cudaError_t mlp_upload(const float* prm, MlpDevWeights* w, cudaStream_t st);

// ---- solver side (learned.cu)
// Per-row features of the current renew, normalised, BF16 [m x HELP_MLP_IN]:
//  0 log10 diag(G)_i   1..4 mean / std / min / max of log10 d_j over row i of A
//  5 log2(1 + row length)   6 log10(D_S,i / diag_i) (0 on pivot rows)
//  7 pivot flag   8 this solve slot's solution in the previous renew, over
//  its RMS (0 if none)   9 / 10 mean / largest |change| of log10 d over the
//  row since the previous renew (0 if none)
// With X null: the raw (unnormalised) FP32 features into R [m x HELP_MLP_IN].
cudaError_t mlp_features(const int* rp, const int* ci, const double* d, const double* diag, const double* dsinv,
                         const int* pivpos, const double* xprev, const double* xprev_sumsq, const double* dprev,
                         int m, const MlpDevWeights* w, __nv_bfloat16* X, float* R, cudaStream_t st);
// dsinv_i *= exp(-clamp(out[i, 0])) on non-pivot rows (FP32 copy too when not null)
cudaError_t mlp_apply_diag(const float* out, const int* pivpos, double* dsinv, float* dsinv32, int m,
                           cudaStream_t st);
// v_i = out[i, 1] * xprev_i
cudaError_t mlp_warm_vector(const float* out, const double* xprev, double* v, int m, cudaStream_t st);

}  // namespace help
