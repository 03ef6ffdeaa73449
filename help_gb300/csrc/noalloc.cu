// (A D^-1 A^T) x without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// runtime's memory pool or under an allocator that forbids new device
// allocations, embedded or real-time paths that must not allocate after
// start-up, or a host process that only ever receives device pointers from
// its caller.  help_adat_matvec_noalloc serves them: the caller passes A (in
// both layouts), d, x and y as device arrays, and the only other memory the
// product needs -- the intermediate t = D^-1 A^T x of n entries -- lives in
// the file-scope device array below.  It is a fixed kNoallocMaxCols doubles
// (8 MiB); every GPU that loads this library holds it until the process
// exits.  The CUDA runtime loads a library's device code lazily by default,
// so the array is reserved by the first call on each device (that call takes
// the 8 MiB of device memory): make it at start-up, before memory is handed
// to the pool that forbids allocation and before any stream capture.
//
// The product is the same two row-gather passes as the backend's
// HELP_OP_ADAT (spmv.cuh), here without a planned row split: every row is
// taken by a group of G lanes sized from the average row length.
#include <cuda_runtime.h>

#include <climits>

#include "../../include/help_gpu.h"
#include "common.cuh"
#include "spmv.cuh"

namespace help {
namespace {

constexpr int kNoallocMaxCols = 1 << 20;  // largest n: 1,048,576 columns (8 MiB of doubles)
constexpr int kNoallocThreads = 256;

// Shared by every call on a device; holds the last call's intermediate t.
__device__ __align__(256) double g_noalloc_t[kNoallocMaxCols];

// Device address of g_noalloc_t on `dev` (the current device) and its SM
// count.  In host code the symbol's name is only a host-side stand-in, so the
// address is asked of the runtime on every call: after a cudaDeviceReset or
// in another context on the same ordinal the module is loaded again, possibly
// at another address, so a cached pointer could go stale.  Once the module is
// loaded the lookup allocates nothing and costs well under a microsecond.
int setup_device(int dev, double** t, int* num_sms) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_t);
    if (e != cudaSuccess) return HELP_E_CUDA;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return HELP_E_CUDA;
    *t = static_cast<double*>(p);
    *num_sms = sms;
    return HELP_OK;
}

int group_for(long long nnz, int rows) {
    const double avg = rows > 0 ? (double)nnz / rows : 0.0;
    int g = 2;
    while (g < 32 && g * 8 < avg) g *= 2;
    return g;
}

SpmvView<double> whole_rows(int rows, int G, const int* ptr, const int* idx, const double* val) {
    SpmvView<double> v;
    v.rows = rows;
    v.G = G;
    v.short_max = INT_MAX;  // no planned split: every row is a group's
    v.n_med = 0;
    v.n_long = 0;
    v.ptr = ptr;
    v.idx = idx;
    v.val = val;
    v.med_rows = nullptr;
    v.long_rows = nullptr;
    return v;
}

// t_j = (A^T x)_j / d_j
__global__ void __launch_bounds__(kNoallocThreads)
    k_noalloc_at(const SpmvView<double> M, const double* __restrict__ x, const double* __restrict__ d,
                 double* __restrict__ t) {
    __shared__ double red[kNoallocThreads];
    spmv_rows<double>(M, [&](int i) { return ld_ro(x + i); }, [&](int j, double s) { t[j] = s / d[j]; }, red);
}

// y_i = (A t)_i
__global__ void __launch_bounds__(kNoallocThreads)
    k_noalloc_a(const SpmvView<double> M, const double* __restrict__ t, double* __restrict__ y) {
    __shared__ double red[kNoallocThreads];
    spmv_rows<double>(M, [&](int j) { return ld_ro(t + j); }, [&](int i, double s) { y[i] = s; }, red);
}

}  // namespace
}  // namespace help

extern "C" int help_adat_matvec_noalloc(int32_t m, int32_t n, int64_t nnz, const int32_t* row_ptr,
                                        const int32_t* col_ind, const double* val, const int32_t* col_ptr,
                                        const int32_t* row_ind, const double* val_t, const double* d,
                                        const double* x, double* y, void* stream) {
    using namespace help;
    if (m <= 0 || n <= 0 || nnz < 0 || !row_ptr || !col_ind || !val || !col_ptr || !row_ind || !val_t || !d || !x ||
        !y)
        return HELP_E_ARG;
    if (n > kNoallocMaxCols) return HELP_E_ARG;  // the scratch array holds at most kNoallocMaxCols entries
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HELP_E_CUDA;
    double* t = nullptr;
    int sms = 0;
    const int rc = setup_device(dev, &t, &sms);
    if (rc != HELP_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int blocks = sms * 8;
    // every t_j is written by the first pass, so the array needs no clearing
    k_noalloc_at<<<blocks, kNoallocThreads, 0, st>>>(whole_rows(n, group_for(nnz, n), col_ptr, row_ind, val_t), x, d, t);
    k_noalloc_a<<<blocks, kNoallocThreads, 0, st>>>(whole_rows(m, group_for(nnz, m), row_ptr, col_ind, val), t, y);
    return cudaGetLastError() == cudaSuccess ? HELP_OK : HELP_E_CUDA;
}
