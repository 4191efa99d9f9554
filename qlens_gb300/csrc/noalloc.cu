// noalloc.cu -- SPD solve + log determinant that allocates no memory.
//
// Some callers cannot call cudaMalloc: a host application that owns the GPU's
// memory budget and hands this library only the buffers it has already
// allocated (through its own pool allocator), or a latency-critical loop
// where cudaMalloc / cudaFree would stall the device with their implicit
// synchronisation.  For them qlp_spd_solve_logdet_noalloc factors an SPD
// matrix they pass in device memory, writes log det and the solution of
// F s = D into their output buffers, and uses as scratch only the file-scope
// device array below, which exists once per GPU for the life of the process.
//
// This is the dense inversion step of the likelihood (the FP64 Cholesky,
// log det and triangular solves that qlp_eval runs on F, see linalg.cu and
// chol.cuh) fused into one single-block kernel that works on a copy of F in
// the static scratch instead of an allocated workspace.
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include "qlpix_internal.h"

namespace qlpix {

// Largest matrix the no-allocation entry point accepts.
#define QLP_NOALLOC_MAX_N 512

// The scratch: the working copy of F (its Cholesky factor after the call),
// the forward-substitution vector and a status word.  Every GPU that loads
// the library holds these ~2.1 MB until the process exits.
struct NoAllocScratch {
    double factor[QLP_NOALLOC_MAX_N * QLP_NOALLOC_MAX_N];
    double y[QLP_NOALLOC_MAX_N];
    int status;
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Single block: copy the lower triangle of F, right-looking Cholesky, log det
// = 2 sum log L_ii, then L y = D and L^T s = y.  A pivot d <= 0 is recorded in
// the status (the first one's index + 1) and the factorisation continues with
// sqrt(|d|), so the call always ends; the reference's Cholesky_dcmp_packed
// (pixelgrid.cpp:17071-17105) flags only d < 0 and would divide by a zero
// pivot.  After a recorded pivot the outputs are not meaningful.
__global__ void __launch_bounds__(1024) k_spd_solve_logdet_noalloc(NoAllocScratch* __restrict__ scr,
                                                                   const double* __restrict__ F, int n, int ld,
                                                                   const double* __restrict__ D,
                                                                   double* __restrict__ s, double* __restrict__ logdet)
{
    __shared__ double red[32];
    double* A = scr->factor;
    const int tid = threadIdx.x, nth = blockDim.x;
    // status starts at zero on every call: the array keeps the previous call's contents
    if (tid == 0) scr->status = 0;
    for (int idx = tid; idx < n * n; idx += nth) {
        const int r = idx / n, c = idx - r * n;
        A[idx] = (c <= r) ? F[(size_t)r * ld + c] : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < n; j++) {
        if (tid == 0) {
            const double d = A[j * n + j];
            if (d <= 0 && scr->status == 0) scr->status = j + 1;
            A[j * n + j] = sqrt(fabs(d));
        }
        __syncthreads();
        const double djj = A[j * n + j];
        for (int i = j + 1 + tid; i < n; i += nth) A[i * n + j] /= djj;
        __syncthreads();
        const int rem = n - j - 1;
        for (int idx = tid; idx < rem * rem; idx += nth) {
            const int i = j + 1 + idx / rem, c = j + 1 + idx % rem;
            if (c <= i) A[i * n + c] -= A[i * n + j] * A[c * n + j];
        }
        __syncthreads();
    }
    // log det
    double acc = 0;
    for (int i = tid; i < n; i += nth) acc += log(fabs(A[i * n + i]));
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
        double t = 0;
        for (int w = 0; w < (nth >> 5); w++) t += red[w];
        *logdet = 2 * t;
    }
    // forward: L y = D (column-oriented)
    double* y = scr->y;
    for (int i = tid; i < n; i += nth) y[i] = D[i];
    __syncthreads();
    for (int c = 0; c < n; c++) {
        if (tid == 0) y[c] /= A[c * n + c];
        __syncthreads();
        const double yc = y[c];
        for (int i = c + 1 + tid; i < n; i += nth) y[i] -= A[i * n + c] * yc;
        __syncthreads();
    }
    // backward: L^T s = y (row c of L^T is column c of L)
    for (int c = n - 1; c >= 0; c--) {
        if (tid == 0) y[c] /= A[c * n + c];
        __syncthreads();
        const double yc = y[c];
        for (int i = tid; i < c; i += nth) y[i] -= A[c * n + i] * yc;
        __syncthreads();
    }
    for (int i = tid; i < n; i += nth) s[i] = y[i];
}

// Device address of the scratch, looked up once per device (on the first call
// made with that device current) and kept: a cudaDeviceReset by the caller
// would leave it stale, so the entry point is not for use after one.
static std::mutex g_noalloc_mu;
static NoAllocScratch* g_noalloc_ptr[64];
static bool g_noalloc_ready[64];

static int noalloc_scratch_for_current_device(NoAllocScratch** out, std::string& err)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        err = "no current CUDA device";
        return QLP_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ready[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            err = std::string("cudaGetSymbolAddress failed for the no-allocation scratch: ") + cudaGetErrorString(e);
            return QLP_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = reinterpret_cast<NoAllocScratch*>(p);
        g_noalloc_ready[dev] = true;
    }
    *out = g_noalloc_ptr[dev];
    return QLP_OK;
}

int spd_solve_logdet_noalloc(const double* F, int n, int ld, const double* D, double* s, double* logdet,
                             void* stream, std::string& err)
{
    if (n < 1 || n > QLP_NOALLOC_MAX_N) {
        err = "qlp_spd_solve_logdet_noalloc: n=" + std::to_string(n) + " outside 1.." +
              std::to_string(QLP_NOALLOC_MAX_N) + " (the size of the static scratch)";
        return QLP_ERR_ARG;
    }
    if (ld < n || !F || !D || !s || !logdet) {
        err = "qlp_spd_solve_logdet_noalloc: null pointer or ld < n";
        return QLP_ERR_ARG;
    }
    NoAllocScratch* scr = nullptr;
    int rc = noalloc_scratch_for_current_device(&scr, err);
    if (rc != QLP_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    k_spd_solve_logdet_noalloc<<<1, 1024, 0, st>>>(scr, F, n, ld, D, s, logdet);
    count_launches(1);
    // the status word follows the kernel on the same stream; one wait for both
    int status = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyFromSymbolAsync(&status, g_noalloc_scratch, sizeof(int), offsetof(NoAllocScratch, status),
                                      cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("qlp_spd_solve_logdet_noalloc: ") + cudaGetErrorString(e);
        return QLP_ERR_CUDA;
    }
    if (status != 0) {
        err = "qlp_spd_solve_logdet_noalloc: matrix not positive definite (pivot " + std::to_string(status - 1) + ")";
        return QLP_ERR_NOT_SPD;
    }
    return QLP_OK;
}

}  // namespace qlpix
