// C ABI of the learned part: a model object (parameters, Adam state,
// training buffers) and its forward / gradient / training-step calls.  The
// solver attaches a model with help_pcg_attach_mlp (api.cu).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/help_gpu.h"
#include "context.h"
#include "guard.h"
#include "mlp.h"

struct help_mlp {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    help::DevMem prm, m1, m2, grad, w;          // FP32 parameters, Adam moments, gradient, device weights
    help::DevMem out, g3, h1, h2, lpart, gpart;  // training buffers (grown with the rows)
    int step = 0;
};

namespace {

int mfail(help_mlp* m, int code, const std::string& msg) {
    if (m) m->err = msg;
    return code;
}

#define MCK(x)                                                                                     \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess) return mfail(mlp, HELP_E_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

int ensure_rows(help_mlp* mlp, long long rows) {
    MCK(mlp->out.ensure(sizeof(float) * HELP_MLP_OUT * (size_t)rows));
    MCK(mlp->g3.ensure(sizeof(float) * HELP_MLP_OUT * (size_t)rows));
    MCK(mlp->h1.ensure(2 * HELP_MLP_HIDDEN * (size_t)rows));
    MCK(mlp->h2.ensure(2 * HELP_MLP_HIDDEN * (size_t)rows));
    MCK(mlp->gpart.ensure(sizeof(float) * help::kMlpGradParams * (size_t)help::mlp_blocks(rows, mlp->num_sms)));
    MCK(mlp->lpart.ensure(sizeof(double) * 2 * help::kMlpLossBlocks));
    return HELP_OK;
}

// forward (keeping activations) + loss + gradient; loss on the host
int loss_grad(help_mlp* mlp, const void* x, const float* t, const float* wt, long long rows, double* loss) {
    if (rows <= 0 || !x || !t || !wt) return mfail(mlp, HELP_E_ARG, "mlp: empty batch or null pointer");
    int rc = ensure_rows(mlp, rows);
    if (rc) return rc;
    const auto* X = static_cast<const __nv_bfloat16*>(x);
    auto* W = mlp->w.as<help::MlpDevWeights>();
    MCK(help::mlp_forward(X, rows, W, mlp->out.as<float>(), mlp->h1.as<__nv_bfloat16>(), mlp->h2.as<__nv_bfloat16>(),
                          mlp->num_sms, mlp->stream));
    MCK(help::mlp_loss_grad(X, rows, W, mlp->out.as<float>(), t, wt, mlp->g3.as<float>(), mlp->h1.as<__nv_bfloat16>(),
                            mlp->h2.as<__nv_bfloat16>(), mlp->lpart.as<double>(), mlp->gpart.as<float>(),
                            mlp->grad.as<float>(), mlp->num_sms, mlp->stream));
    if (loss) {
        std::vector<double> lp(help::kMlpLossBlocks);
        MCK(cudaMemcpyAsync(lp.data(), mlp->lpart.p, sizeof(double) * lp.size(), cudaMemcpyDeviceToHost, mlp->stream));
        MCK(cudaStreamSynchronize(mlp->stream));
        double s = 0.0;
        for (double v : lp) s += v;
        *loss = s;
    }
    return HELP_OK;
}

}  // namespace

extern "C" {

static int help_mlp_create_body(int32_t device, help_mlp** out) {
    if (!out) return HELP_E_ARG;
    *out = nullptr;
    help_mlp* mlp = new help_mlp();
    mlp->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&mlp->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&mlp->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = mlp->prm.ensure(sizeof(float) * HELP_MLP_PARAMS);
    if (e == cudaSuccess) e = mlp->m1.ensure(sizeof(float) * HELP_MLP_PARAMS);
    if (e == cudaSuccess) e = mlp->m2.ensure(sizeof(float) * HELP_MLP_PARAMS);
    if (e == cudaSuccess) e = mlp->grad.ensure(sizeof(float) * HELP_MLP_PARAMS);
    if (e == cudaSuccess) e = mlp->w.ensure(sizeof(help::MlpDevWeights));
    if (e == cudaSuccess) e = cudaMemset(mlp->prm.p, 0, sizeof(float) * HELP_MLP_PARAMS);
    if (e == cudaSuccess) e = cudaMemset(mlp->w.p, 0, sizeof(help::MlpDevWeights));
    if (e == cudaSuccess) e = help::mlp_configure();
    if (e != cudaSuccess) {
        help_mlp_free(mlp);
        return HELP_E_CUDA;
    }
    *out = mlp;
    return HELP_OK;
}

int help_mlp_create(int32_t device, help_mlp** out) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_create_body(device, out); });
}

static int help_mlp_free_body(help_mlp* mlp) {
    if (!mlp) return HELP_E_ARG;
    cudaSetDevice(mlp->device);
    for (help::DevMem* d : {&mlp->prm, &mlp->m1, &mlp->m2, &mlp->grad, &mlp->w, &mlp->out, &mlp->g3, &mlp->h1,
                            &mlp->h2, &mlp->lpart, &mlp->gpart})
        d->release();
    if (mlp->stream) cudaStreamDestroy(mlp->stream);
    delete mlp;
    return HELP_OK;
}

int help_mlp_free(help_mlp* mlp) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_free_body(mlp); });
}

const char* help_mlp_last_error(const help_mlp* mlp) { return mlp ? mlp->err.c_str() : "null model"; }

static int help_mlp_set_params_body(help_mlp* mlp, const float* params) {
    if (!mlp || !params) return HELP_E_ARG;
    for (int j = 0; j < HELP_MLP_PARAMS; ++j)
        if (!std::isfinite(params[j])) return mfail(mlp, HELP_E_NUMERIC, "mlp: non-finite parameter");
    MCK(cudaSetDevice(mlp->device));
    MCK(cudaMemcpyAsync(mlp->prm.p, params, sizeof(float) * HELP_MLP_PARAMS, cudaMemcpyHostToDevice, mlp->stream));
    MCK(cudaMemsetAsync(mlp->m1.p, 0, sizeof(float) * HELP_MLP_PARAMS, mlp->stream));
    MCK(cudaMemsetAsync(mlp->m2.p, 0, sizeof(float) * HELP_MLP_PARAMS, mlp->stream));
    MCK(help::mlp_upload(mlp->prm.as<float>(), mlp->w.as<help::MlpDevWeights>(), mlp->stream));
    MCK(cudaStreamSynchronize(mlp->stream));
    mlp->step = 0;
    return HELP_OK;
}

int help_mlp_set_params(help_mlp* mlp, const float* params) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_set_params_body(mlp, params); });
}

static int help_mlp_get_params_body(help_mlp* mlp, float* params) {
    if (!mlp || !params) return HELP_E_ARG;
    MCK(cudaSetDevice(mlp->device));
    MCK(cudaMemcpyAsync(params, mlp->prm.p, sizeof(float) * HELP_MLP_PARAMS, cudaMemcpyDeviceToHost, mlp->stream));
    MCK(cudaStreamSynchronize(mlp->stream));
    return HELP_OK;
}

int help_mlp_get_params(help_mlp* mlp, float* params) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_get_params_body(mlp, params); });
}

static int help_mlp_forward_body(help_mlp* mlp, const void* x, int64_t rows, float* out, void* stream) {
    if (!mlp || !x || !out || rows < 0) return HELP_E_ARG;
    MCK(cudaSetDevice(mlp->device));
    MCK(help::mlp_forward(static_cast<const __nv_bfloat16*>(x), rows, mlp->w.as<help::MlpDevWeights>(), out, nullptr,
                          nullptr, mlp->num_sms, static_cast<cudaStream_t>(stream)));
    return HELP_OK;
}

int help_mlp_forward(help_mlp* mlp, const void* x, int64_t rows, float* out, void* stream) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_forward_body(mlp, x, rows, out, stream); });
}

static int help_mlp_loss_grad_body(help_mlp* mlp, const void* x, const float* target, const float* weight, int64_t rows,
                       double* loss, float* grad) {
    if (!mlp) return HELP_E_ARG;
    MCK(cudaSetDevice(mlp->device));
    int rc = loss_grad(mlp, x, target, weight, rows, loss);
    if (rc) return rc;
    if (grad) {
        MCK(cudaMemcpyAsync(grad, mlp->grad.p, sizeof(float) * help::kMlpGradParams, cudaMemcpyDeviceToHost,
                            mlp->stream));
        MCK(cudaStreamSynchronize(mlp->stream));
    }
    return HELP_OK;
}

int help_mlp_loss_grad(help_mlp* mlp, const void* x, const float* target, const float* weight, int64_t rows,
                       double* loss, float* grad) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_loss_grad_body(mlp, x, target, weight, rows, loss, grad); });
}

static int help_mlp_train_step_body(help_mlp* mlp, const void* x, const float* target, const float* weight, int64_t rows,
                        float lr, double* loss) {
    if (!mlp || !(lr > 0.f)) return HELP_E_ARG;
    MCK(cudaSetDevice(mlp->device));
    int rc = loss_grad(mlp, x, target, weight, rows, loss);
    if (rc) return rc;
    mlp->step += 1;
    MCK(help::mlp_adam(mlp->prm.as<float>(), mlp->m1.as<float>(), mlp->m2.as<float>(), mlp->grad.as<float>(), lr,
                       mlp->step, mlp->w.as<help::MlpDevWeights>(), mlp->stream));
    MCK(cudaStreamSynchronize(mlp->stream));
    return HELP_OK;
}

int help_mlp_train_step(help_mlp* mlp, const void* x, const float* target, const float* weight, int64_t rows,
                        float lr, double* loss) {
    return c_guard(HELP_E_NOMEM, [&] { return help_mlp_train_step_body(mlp, x, target, weight, rows, lr, loss); });
}

}  // extern "C"

// Device weights of a model (for the solver in api.cu).
const help::MlpDevWeights* help_mlp_device_weights(const help_mlp* mlp) {
    return mlp ? mlp->w.as<help::MlpDevWeights>() : nullptr;
}
int help_mlp_device(const help_mlp* mlp) { return mlp ? mlp->device : -1; }
