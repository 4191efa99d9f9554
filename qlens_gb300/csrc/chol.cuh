// chol.cuh -- blocked dense Cholesky (lower), log det and triangular solves,
// templated on the factor's element type (double for the plain path, float
// for the mixed-precision path).  Vectors are always FP64.
//
// Reference: QLens::Cholesky_dcmp_packed (pixelgrid.cpp:17071-17105; a
// negative pivot is flagged and sqrt(|d|) used), Cholesky_logdet_lower_packed
// (17201-17210), Cholesky_solve_lower_packed (17230-17246).  The reference
// factors a packed triangle row by row; here the same factorisation runs as a
// right-looking blocked algorithm on 64x64 tiles: factor the diagonal tile,
// solve the tiles below it, update the trailing lower triangle.  Sizes come
// from the device-side GridState (M active cells, padded to 64 with identity).
#pragma once
#include "qlpix_internal.h"

namespace qlpix {

#define CB 64

__device__ __forceinline__ int cpad64(int M) { return (M + 63) & ~63; }

__device__ __forceinline__ void tri_index(int t, int& bi, int& bj)
{
    int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) i++;
    while (i * (i + 1) / 2 > t) i--;
    bi = i;
    bj = t - i * (i + 1) / 2;
}

// Factor the 64x64 diagonal tile in shared memory (two barriers per pivot:
// scaled pivot column, then the rank-1 update), and, when Linv is given,
// write the inverse of the factor: columns of L X = I by forward
// substitution, four threads per column.
template <typename T>
__global__ void __launch_bounds__(256) k_potrf_t(T* __restrict__ A, int ld, int k, GridState* gs, int which,
                                                 T* __restrict__ Linv)
{
    __shared__ T S[CB][CB + 1];
    __shared__ T colj[CB];
    const int nblk = cpad64(gs->M) / CB;
    if (k >= nblk) return;
    const int o = k * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        S[r][c] = (c <= r) ? A[(size_t)(o + r) * ld + o + c] : T(0);
    }
    __syncthreads();
    for (int j = 0; j < CB; j++) {
        if (threadIdx.x >= j && threadIdx.x < CB) {
            const T d = S[j][j];
            if (threadIdx.x == j && d < 0) {
                // Cholesky_dcmp_packed continues with sqrt(|d|) and flags the matrix
                int* flag = which ? &gs->not_spd_R : &gs->not_spd_F;
                if (*flag == 0) *flag = o + j + 1;
            }
            const T sd = sqrt(fabs(d));
            colj[threadIdx.x] = (threadIdx.x == j) ? sd : S[threadIdx.x][j] / sd;
        }
        __syncthreads();
        {
            const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
            for (int i = j + 1 + ty; i < CB; i += 16) {
                const T ci = colj[i];
                for (int c = j + 1 + tx; c <= i; c += 16) S[i][c] -= ci * colj[c];
            }
        }
        if (threadIdx.x >= j && threadIdx.x < CB) S[threadIdx.x][j] = colj[threadIdx.x];
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        if (c <= r) A[(size_t)(o + r) * ld + o + c] = S[r][c];
    }
    if (Linv == nullptr) return;
    // X = L^-1 column by column; thread group g (4 lanes) owns column j = g.
    __shared__ T X[CB][CB + 1];
    const int j = threadIdx.x >> 2, q = threadIdx.x & 3;
    for (int i = 0; i < CB; i++) {
        T part = 0;
        if (i > j)
            for (int m = j + q; m < i; m += 4) part += S[i][m] * X[m][j];
        part += __shfl_xor_sync(0xffffffffu, part, 1);
        part += __shfl_xor_sync(0xffffffffu, part, 2);
        if (q == 0) X[i][j] = (i < j) ? T(0) : (i == j ? T(1) / S[i][i] : -part / S[i][i]);
        __syncwarp();
    }
    __syncthreads();
    T* Lk = Linv + (size_t)k * CB * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) Lk[idx] = X[idx / CB][idx % CB];
}

// ---------------------------------------------------------------------------
// FP32 kernels with the factor rows in registers.
// ---------------------------------------------------------------------------

// One warp factors the 64x64 diagonal tile: lane l holds rows l and l+32 in
// registers; pivot and column values travel by shuffle.  Fully unrolled.
static __global__ void __launch_bounds__(32) k_potrf_warp(float* __restrict__ A, int ld, int k, GridState* gs, int which)
{
    const int nblk = cpad64(gs->M) / CB;
    if (k >= nblk) return;
    const int o = k * CB;
    const int lane = threadIdx.x;
    float a0[CB], a1[CB];
    const float* r0 = A + (size_t)(o + lane) * ld + o;
    const float* r1 = A + (size_t)(o + lane + 32) * ld + o;
    #pragma unroll
    for (int c = 0; c < CB; c++) {
        a0[c] = (c <= lane) ? r0[c] : 0.f;
        a1[c] = (c <= lane + 32) ? r1[c] : 0.f;
    }
    #pragma unroll
    for (int j = 0; j < CB; j++) {
        const float dv = __shfl_sync(0xffffffffu, (j < 32) ? a0[j] : a1[j], j & 31);
        if (lane == 0 && dv < 0.f) {
            int* flag = which ? &gs->not_spd_R : &gs->not_spd_F;
            if (*flag == 0) *flag = o + j + 1;
        }
        const float sd = sqrtf(fabsf(dv));
        const float rinv = 1.0f / sd;
        if (j < 32) {
            if (lane > j) a0[j] *= rinv;
            else if (lane == j) a0[j] = sd;
        }
        if (lane + 32 > j) a1[j] *= rinv;
        else if (lane + 32 == j) a1[j] = sd;
        #pragma unroll
        for (int c = j + 1; c < CB; c++) {
            const float vc = __shfl_sync(0xffffffffu, (c < 32) ? a0[j] : a1[j], c & 31);
            if (c < 32 && c <= lane) a0[c] -= a0[j] * vc;
            if (c <= lane + 32) a1[c] -= a1[j] * vc;
        }
    }
    float* w0 = A + (size_t)(o + lane) * ld + o;
    float* w1 = A + (size_t)(o + lane + 32) * ld + o;
    #pragma unroll
    for (int c = 0; c < CB; c++) {
        if (c <= lane) w0[c] = a0[c];
        if (c <= lane + 32) w1[c] = a1[c];
    }
}

// Tiles below the diagonal: X L_kk^T = A_ik by forward substitution, one
// thread per row of the tile with the row in registers, L_kk in shared memory.
static __global__ void __launch_bounds__(CB) k_trsm_rows(float* __restrict__ A, int ld, int k, const GridState* __restrict__ gs)
{
    __shared__ float Lk[CB][CB + 1];
    const int nblk = cpad64(gs->M) / CB;
    const int i = k + 1 + blockIdx.x;
    if (i >= nblk) return;
    const int o = k * CB, ro = i * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        const int r = idx / CB, c = idx % CB;
        Lk[r][c] = (c <= r) ? A[(size_t)(o + r) * ld + o + c] : 0.f;
    }
    float x[CB];
    float* row = A + (size_t)(ro + threadIdx.x) * ld + o;
    #pragma unroll
    for (int c = 0; c < CB; c++) x[c] = row[c];
    __syncthreads();
    #pragma unroll
    for (int c = 0; c < CB; c++) {
        float a0 = x[c], a1 = 0.f, a2 = 0.f, a3 = 0.f;   // four independent chains
        #pragma unroll
        for (int m = 0; m + 3 < c; m += 4) {
            a0 -= x[m] * Lk[c][m];
            a1 -= x[m + 1] * Lk[c][m + 1];
            a2 -= x[m + 2] * Lk[c][m + 2];
            a3 -= x[m + 3] * Lk[c][m + 3];
        }
        #pragma unroll
        for (int m = c & ~3; m < c; m++) a0 -= x[m] * Lk[c][m];
        x[c] = ((a0 + a1) + (a2 + a3)) / Lk[c][c];
    }
    #pragma unroll
    for (int c = 0; c < CB; c++) row[c] = x[c];
}

// Inverses of all diagonal factors at once (after the factorisation, off its
// critical path): thread t of block k computes column t of L_kk^-1.
template <typename T>
__global__ void __launch_bounds__(CB) k_diag_inverse(const T* __restrict__ A, int ld, const GridState* __restrict__ gs,
                                                     T* __restrict__ Linv)
{
    __shared__ T Lk[CB][CB + 1];
    const int nblk = cpad64(gs->M) / CB;
    const int k = blockIdx.x;
    if (k >= nblk) return;
    const int o = k * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        const int r = idx / CB, c = idx % CB;
        Lk[r][c] = (c <= r) ? A[(size_t)(o + r) * ld + o + c] : T(0);
    }
    __syncthreads();
    const int t = threadIdx.x;
    T x[CB];
    #pragma unroll
    for (int i = 0; i < CB; i++) {
        T acc = (i == t) ? T(1) : T(0);
        #pragma unroll
        for (int m = 0; m < i; m++) acc -= Lk[i][m] * x[m];
        x[i] = (i < t) ? T(0) : acc / Lk[i][i];
    }
    T* Lo = Linv + (size_t)k * CB * CB;
    #pragma unroll
    for (int i = 0; i < CB; i++) Lo[i * CB + t] = x[i];
}

// Tiles below the diagonal: X = A_ik L_kk^-T = A_ik Linv^T, a 64x64x64 GEMM
// per block row (the triangular solve through the explicit inverse of the
// small diagonal factor, as blocked GPU Cholesky codes commonly do).
template <typename T>
__global__ void __launch_bounds__(256) k_trsm_inv_t(T* __restrict__ A, int ld, int k, const T* __restrict__ Linv,
                                                    const GridState* __restrict__ gs)
{
    __shared__ T Ab[CB][CB + 1];
    __shared__ T Li[CB][CB + 1];
    const int nblk = cpad64(gs->M) / CB;
    const int i = k + 1 + blockIdx.x;
    if (i >= nblk) return;
    const int o = k * CB, ro = i * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        Ab[r][c] = A[(size_t)(ro + r) * ld + o + c];
        Li[r][c] = Linv[(size_t)k * CB * CB + r * CB + c];
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0;
    #pragma unroll 8
    for (int m = 0; m < CB; m++) {
        T ra[4], rb[4];
        #pragma unroll
        for (int u = 0; u < 4; u++) ra[u] = Ab[ty * 4 + u][m];
        #pragma unroll
        for (int v = 0; v < 4; v++) rb[v] = Li[tx * 4 + v][m];
        #pragma unroll
        for (int u = 0; u < 4; u++)
            #pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] += ra[u] * rb[v];
    }
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) A[(size_t)(ro + ty * 4 + u) * ld + o + tx * 4 + v] = acc[u][v];
}

template <typename T>
__global__ void __launch_bounds__(256) k_trsm_t(T* __restrict__ A, int ld, int k, const GridState* __restrict__ gs)
{
    __shared__ T Lk[CB][CB + 1];
    __shared__ T X[CB][CB + 1];
    const int nblk = cpad64(gs->M) / CB;
    const int i = k + 1 + blockIdx.x;
    if (i >= nblk) return;
    const int o = k * CB, ro = i * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        Lk[r][c] = (c <= r) ? A[(size_t)(o + r) * ld + o + c] : T(0);
        X[r][c] = A[(size_t)(ro + r) * ld + o + c];
    }
    __syncthreads();
    for (int c = 0; c < CB; c++) {
        const T dcc = Lk[c][c];
        for (int r = threadIdx.x; r < CB; r += blockDim.x) X[r][c] /= dcc;
        __syncthreads();
        const int rem = CB - c - 1;
        for (int idx = threadIdx.x; idx < CB * rem; idx += blockDim.x) {
            int r = idx / rem, c2 = c + 1 + idx % rem;
            X[r][c2] -= X[r][c] * Lk[c2][c];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        A[(size_t)(ro + r) * ld + o + c] = X[r][c];
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_chol_update_t(T* __restrict__ A, int ld, int k,
                                                       const GridState* __restrict__ gs)
{
    __shared__ T Li[CB][CB + 1];
    __shared__ T Lj[CB][CB + 1];
    const int nblk = cpad64(gs->M) / CB;
    int ti, tj;
    tri_index(blockIdx.x, ti, tj);
    const int i = k + 1 + ti, j = k + 1 + tj;
    if (i >= nblk) return;
    const int o = k * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        Li[r][c] = A[(size_t)(i * CB + r) * ld + o + c];
        Lj[r][c] = A[(size_t)(j * CB + r) * ld + o + c];
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0;
    #pragma unroll 8
    for (int kk = 0; kk < CB; kk++) {
        T ra[4], rb[4];
        #pragma unroll
        for (int u = 0; u < 4; u++) ra[u] = Li[ty * 4 + u][kk];
        #pragma unroll
        for (int v = 0; v < 4; v++) rb[v] = Lj[tx * 4 + v][kk];
        #pragma unroll
        for (int u = 0; u < 4; u++)
            #pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] += ra[u] * rb[v];
    }
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) {
            size_t off = (size_t)(i * CB + ty * 4 + u) * ld + j * CB + tx * 4 + v;
            A[off] -= acc[u][v];
        }
}

// Linv: (M_cap/64) x 64 x 64 storage for the inverses of the diagonal
// factors; the trsm step and the triangular solves use them.
template <typename T>
int launch_cholesky_t(T* A, int ld, int M_cap, const GridState* gs, int which, cudaStream_t st, T* Linv)
{
    const int nbm = (M_cap + CB - 1) / CB;
    int n = 0;
    for (int k = 0; k < nbm; k++) {
        const int rem = nbm - k - 1;
        k_potrf_t<T><<<1, 256, 0, st>>>(A, ld, k, const_cast<GridState*>(gs), which, Linv);
        n++;
        if (rem > 0) {
            k_trsm_inv_t<T><<<rem, 256, 0, st>>>(A, ld, k, Linv, gs);
            k_chol_update_t<T><<<rem * (rem + 1) / 2, 256, 0, st>>>(A, ld, k, gs);
            n += 2;
        }
    }
    count_launches(n);
    return n;
}

template <typename T>
__global__ void __launch_bounds__(1024) k_logdet_t(const T* __restrict__ A, int ld, const GridState* __restrict__ gs,
                                                   EvalOut* out, int which)
{
    __shared__ double red[32];
    const int M = gs->M;
    double acc = 0;
    for (int i = threadIdx.x; i < M; i += blockDim.x) acc += log(fabs((double)A[(size_t)i * ld + i]));
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[k];
        if (which) out->logdet_R = 2 * t;
        else out->logdet_F = 2 * t;
    }
}

// F z = r with the Cholesky factor in A (lower) and the inverses of its
// 64x64 diagonal blocks (Linv), one block of 1024 threads.  The arithmetic
// type is T (float for the mixed path, double for the plain path); r and z
// are FP64 in global memory, y and z are staged in shared memory as T.
//   forward  y_k = Linv_k (r_k - sum_{j<k} L_kj y_j)
//   backward z_k = Linv_k^T (y_k - sum_{j>k} L_jk^T z_j)
// Dynamic shared memory: solve_smem_bytes<T>(M_cap).
template <typename T>
__host__ __device__ __forceinline__ size_t solve_smem_bytes(int M_cap)
{
    return sizeof(T) * ((size_t)2 * M_cap + 2 * CB + 16 * (CB + 1));
}

template <typename T>
__global__ void __launch_bounds__(1024) k_solve_t(const T* __restrict__ A, int ld, const T* __restrict__ Linv,
                                                  const GridState* __restrict__ gs, const double* __restrict__ r,
                                                  double* __restrict__ zout, int M_cap)
{
    extern __shared__ __align__(16) unsigned char sm_solve_raw[];
    T* y = reinterpret_cast<T*>(sm_solve_raw);
    T* z = y + M_cap;
    T* t = z + M_cap;                 // [CB] block right-hand side
    T* part = t + 2 * CB;             // [16][CB+1]
    const int Mp = cpad64(gs->M);
    const int nblk = Mp / CB;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < Mp; i += blockDim.x) { y[i] = (T)r[i]; z[i] = 0; }
    __syncthreads();
    // ---- forward ----
    for (int kb = 0; kb < nblk; kb++) {
        const int o = kb * CB;
        for (int h = 0; h < 2; h++) {
            const int row = warp * 2 + h;
            const T* Ar = A + (size_t)(o + row) * ld;
            T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
            int c = lane;
            for (; c + 224 < o; c += 256) {
                const T v0 = Ar[c], v1 = Ar[c + 32], v2 = Ar[c + 64], v3 = Ar[c + 96];
                const T v4 = Ar[c + 128], v5 = Ar[c + 160], v6 = Ar[c + 192], v7 = Ar[c + 224];
                a0 += v0 * y[c] + v4 * y[c + 128];
                a1 += v1 * y[c + 32] + v5 * y[c + 160];
                a2 += v2 * y[c + 64] + v6 * y[c + 192];
                a3 += v3 * y[c + 96] + v7 * y[c + 224];
            }
            for (; c < o; c += 32) a0 += Ar[c] * y[c];
            T acc = (a0 + a1) + (a2 + a3);
            for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
            if (lane == 0) t[row] = y[o + row] - acc;
        }
        __syncthreads();
        {   // y_k = Linv_k t: 16 threads per row
            const int row = tid >> 4, q = tid & 15;
            const T* Lr = Linv + (size_t)kb * CB * CB + row * CB;
            T acc = 0;
            for (int m = q; m <= row; m += 16) acc += Lr[m] * t[m];
            for (int off = 8; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
            if (q == 0) y[o + row] = acc;
        }
        __syncthreads();
    }
    // ---- backward ----
    for (int kb = nblk - 1; kb >= 0; kb--) {
        const int o = kb * CB, e = o + CB;
        {
            const int c = tid & 63, tt = tid >> 6;
            T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
            int rr = e + tt;
            for (; rr + 48 < Mp; rr += 64) {
                const T v0 = A[(size_t)rr * ld + o + c];
                const T v1 = A[(size_t)(rr + 16) * ld + o + c];
                const T v2 = A[(size_t)(rr + 32) * ld + o + c];
                const T v3 = A[(size_t)(rr + 48) * ld + o + c];
                a0 += v0 * z[rr];
                a1 += v1 * z[rr + 16];
                a2 += v2 * z[rr + 32];
                a3 += v3 * z[rr + 48];
            }
            for (; rr < Mp; rr += 16) a0 += A[(size_t)rr * ld + o + c] * z[rr];
            part[tt * (CB + 1) + c] = (a0 + a1) + (a2 + a3);
        }
        __syncthreads();
        if (tid < CB) {
            T acc = 0;
            for (int q = 0; q < 16; q++) acc += part[q * (CB + 1) + tid];
            t[tid] = y[o + tid] - acc;
        }
        __syncthreads();
        {   // z_k = Linv_k^T t: column c of Linv, 16 threads per column
            const int c = tid >> 4, q = tid & 15;
            const T* Lk = Linv + (size_t)kb * CB * CB;
            T acc = 0;
            for (int m = c + q; m < CB; m += 16) acc += Lk[m * CB + c] * t[m];
            for (int off = 8; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
            if (q == 0) z[o + c] = acc;
        }
        __syncthreads();
    }
    for (int i = tid; i < Mp; i += blockDim.x) zout[i] = (double)z[i];
}

template <typename T>
void solve_init_attributes()
{
    cudaFuncSetAttribute(k_solve_t<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// FP32 blocked Cholesky with the register kernels, then the diagonal inverses.
inline int launch_cholesky_f32(float* A, int ld, int M_cap, const GridState* gs, int which, cudaStream_t st,
                               float* Linv)
{
    const int nbm = (M_cap + CB - 1) / CB;
    int n = 0;
    for (int k = 0; k < nbm; k++) {
        const int rem = nbm - k - 1;
        k_potrf_warp<<<1, 32, 0, st>>>(A, ld, k, const_cast<GridState*>(gs), which);
        n++;
        if (rem > 0) {
            k_trsm_rows<<<rem, CB, 0, st>>>(A, ld, k, gs);
            k_chol_update_t<float><<<rem * (rem + 1) / 2, 256, 0, st>>>(A, ld, k, gs);
            n += 2;
        }
    }
    k_diag_inverse<float><<<nbm, CB, 0, st>>>(A, ld, gs, Linv);
    n++;
    count_launches(n);
    return n;
}

}  // namespace qlpix
