// Residual norms ||b_j - A x_j||_2 with no device allocation.
//
// Some hosts of this library cannot call cudaMalloc while they solve: a FEM
// application that has reserved the whole device memory for its own pool,
// a caller recording its work into a CUDA stream capture (where allocation
// calls are not permitted), or a time-critical loop that must not take the
// implicit device synchronisation an allocation can cause.  For them this
// file offers the FP64 residual check of uchol_residual_norms with every
// buffer supplied by the caller and the only scratch in a fixed-size array
// that the library declares statically on every device that loads it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../../include/uchol_gpu.h"

namespace {

// Scratch: the product A x (n * nrhs doubles) followed by per-block partial
// sums of the squared residual (kBlocks * nrhs doubles).  8 MiB per device,
// held from library load until process exit.
constexpr long long kScratchDoubles = 1 << 20;
constexpr int kBlocks = 128;
constexpr int kMaxColumns = 64;
static __device__ __align__(256) double g_residual_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
CUcontext g_scratch_ctx[kMaxDevices] = {nullptr};   // the context each cached address belongs to
thread_local std::string g_static_error;

struct Fail {
    int code;
    std::string msg;
};

// y += A x from the upper triangle: row entries directly, mirrored entries
// by atomic accumulation.
__global__ void k_upper_product(int n, int nrhs, const int* __restrict__ row_ptr, const int* __restrict__ col,
                                const double* __restrict__ val, const double* __restrict__ x, int ldx,
                                double* __restrict__ y) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int r = warp;
    for (int j = 0; j < nrhs; ++j) {
        const double* xj = x + (long long)j * ldx;
        double* yj = y + (long long)j * n;
        double acc = 0.0;
        for (int p = row_ptr[r] + lane; p < row_ptr[r + 1]; p += 32) {
            const int c = col[p];
            const double v = val[p];
            acc += v * xj[c];
            if (c != r) atomicAdd(&yj[c], v * xj[r]);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) atomicAdd(&yj[r], acc);
    }
}

// Partial sums of (b - y)^2 per block and column, fixed block order.
__global__ void k_residual_partials(int n, int nrhs, const double* __restrict__ b, int ldb,
                                    const double* __restrict__ y, double* __restrict__ partial) {
    __shared__ double red[256];
    for (int j = 0; j < nrhs; ++j) {
        double acc = 0.0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const double d = b[i + (long long)j * ldb] - y[i + (long long)j * n];
            acc += d * d;
        }
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[blockIdx.x + j * gridDim.x] = red[0];
        __syncthreads();
    }
}

__global__ void k_residual_finish(const double* __restrict__ partial, int blocks, int nrhs, double* __restrict__ out) {
    const int j = threadIdx.x;
    if (j >= nrhs) return;
    double s = 0.0;
    for (int k = 0; k < blocks; ++k) s += partial[k + j * blocks];
    out[j] = sqrt(s);
}

// The driver's cuCtxGetCurrent, through the runtime (the library links no driver library).
CUresult current_context(CUcontext* ctx) {
    using Fn = CUresult (*)(CUcontext*);
    static Fn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return CUDA_ERROR_NOT_FOUND;
        fn = reinterpret_cast<Fn>(p);
    }
    return fn(ctx);
}

// Device address of the static array on the current device, looked up once per device and
// context: after a device reset (or under another context) the module is loaded anew and
// the address is looked up again.
double* scratch_on_current_device() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw Fail{UCHOL_CUDA_ERROR, std::string("cudaGetDevice failed: ") + cudaGetErrorString(e)};
    if (dev < 0 || dev >= kMaxDevices) throw Fail{UCHOL_BAD_ARG, "device ordinal out of range"};
    // no context is current yet on a thread that has made no CUDA call: then the lookup below
    // (which makes the device's primary context current) runs, and the context is read after it
    CUcontext ctx = nullptr;
    if (current_context(&ctx) != CUDA_SUCCESS) throw Fail{UCHOL_CUDA_ERROR, "cuCtxGetCurrent failed"};
    std::lock_guard<std::mutex> lk(g_mu);
    if (!ctx || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_residual_scratch);
        if (e != cudaSuccess || !p)
            throw Fail{UCHOL_CUDA_ERROR,
                       std::string("cudaGetSymbolAddress of the static scratch failed: ") + cudaGetErrorString(e)};
        if (current_context(&ctx) != CUDA_SUCCESS || !ctx) throw Fail{UCHOL_CUDA_ERROR, "no current CUDA context"};
        g_scratch_ptr[dev] = static_cast<double*>(p);
        g_scratch_ctx[dev] = ctx;
    }
    return g_scratch_ptr[dev];
}

}  // namespace

extern "C" int uchol_residual_norms_static(int n, int nnz, int nrhs, const int* d_row_ptr, const int* d_col,
                                           const double* d_values, const double* d_b, int ldb, const double* d_x,
                                           int ldx, double* d_norms, void* stream) {
    try {
        if (n < 0 || nnz < 0 || nrhs < 0) throw Fail{UCHOL_BAD_ARG, "negative size"};
        if (nrhs == 0) return UCHOL_OK;
        if (!d_norms || (n > 0 && (!d_row_ptr || !d_b || !d_x)) || (nnz > 0 && (!d_col || !d_values)))
            throw Fail{UCHOL_BAD_ARG, "null device pointer"};
        if (ldb < (n > 0 ? n : 1) || ldx < (n > 0 ? n : 1)) throw Fail{UCHOL_BAD_ARG, "leading dimension smaller than n"};
        if (nrhs > kMaxColumns)
            throw Fail{UCHOL_BAD_ARG, "at most " + std::to_string(kMaxColumns) + " right-hand sides per call"};
        if ((long long)n * nrhs + (long long)kBlocks * nrhs > kScratchDoubles)
            throw Fail{UCHOL_BAD_ARG, "n * nrhs = " + std::to_string((long long)n * nrhs) +
                                          " exceeds the static scratch of this entry point (" +
                                          std::to_string(kScratchDoubles - (long long)kBlocks * nrhs) +
                                          " doubles for this nrhs); use uchol_residual_norms instead"};
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        double* scratch = scratch_on_current_device();
        double* y = scratch;
        double* partial = scratch + (long long)n * nrhs;
        cudaError_t e = cudaMemsetAsync(y, 0, sizeof(double) * (size_t)n * nrhs, st);
        if (e != cudaSuccess) throw Fail{UCHOL_CUDA_ERROR, std::string("clearing the scratch failed: ") + cudaGetErrorString(e)};
        if (n > 0)
            k_upper_product<<<(n + 7) / 8, 256, 0, st>>>(n, nrhs, d_row_ptr, d_col, d_values, d_x, ldx, y);
        k_residual_partials<<<kBlocks, 256, 0, st>>>(n, nrhs, d_b, ldb, y, partial);
        k_residual_finish<<<1, kMaxColumns, 0, st>>>(partial, kBlocks, nrhs, d_norms);
        e = cudaGetLastError();
        if (e != cudaSuccess) throw Fail{UCHOL_CUDA_ERROR, std::string("kernel launch failed: ") + cudaGetErrorString(e)};
        g_static_error.clear();
        return UCHOL_OK;
    } catch (const Fail& f) {
        g_static_error = f.msg;
        return f.code;
    }
}

extern "C" const char* uchol_residual_norms_static_error(void) { return g_static_error.c_str(); }
