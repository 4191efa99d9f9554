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

template <typename T>
__global__ void __launch_bounds__(256) k_potrf_t(T* __restrict__ A, int ld, int k, GridState* gs, int which)
{
    __shared__ T S[CB][CB + 1];
    const int nblk = cpad64(gs->M) / CB;
    if (k >= nblk) return;
    const int o = k * CB;
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        S[r][c] = (c <= r) ? A[(size_t)(o + r) * ld + o + c] : T(0);
    }
    __syncthreads();
    for (int j = 0; j < CB; j++) {
        if (threadIdx.x == 0) {
            T d = S[j][j];
            if (d < 0) {
                int* flag = which ? &gs->not_spd_R : &gs->not_spd_F;
                if (*flag == 0) *flag = o + j + 1;
            }
            S[j][j] = sqrt(fabs(d));
        }
        __syncthreads();
        const T djj = S[j][j];
        for (int i = j + 1 + threadIdx.x; i < CB; i += blockDim.x) S[i][j] /= djj;
        __syncthreads();
        const int rem = CB - j - 1;
        for (int idx = threadIdx.x; idx < rem * rem; idx += blockDim.x) {
            int i = j + 1 + idx / rem, c = j + 1 + idx % rem;
            if (c <= i) S[i][c] -= S[i][j] * S[c][j];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < CB * CB; idx += blockDim.x) {
        int r = idx / CB, c = idx % CB;
        if (c <= r) A[(size_t)(o + r) * ld + o + c] = S[r][c];
    }
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

template <typename T>
int launch_cholesky_t(T* A, int ld, int M_cap, const GridState* gs, int which, cudaStream_t st)
{
    const int nbm = (M_cap + CB - 1) / CB;
    int n = 0;
    for (int k = 0; k < nbm; k++) {
        k_potrf_t<T><<<1, 256, 0, st>>>(A, ld, k, const_cast<GridState*>(gs), which);
        n++;
        const int rem = nbm - k - 1;
        if (rem > 0) {
            k_trsm_t<T><<<rem, 256, 0, st>>>(A, ld, k, gs);
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

// F z = r with the Cholesky factor in A (lower): blocked forward and backward
// substitution in one block; r, z, y are FP64.
template <typename T>
__global__ void __launch_bounds__(1024) k_solve_t(const T* __restrict__ A, int ld, const GridState* __restrict__ gs,
                                                  const double* __restrict__ r, double* __restrict__ z, double* y)
{
    __shared__ double part[16][CB + 1];
    const int Mp = cpad64(gs->M);
    const int nblk = Mp / CB;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < Mp; i += blockDim.x) y[i] = r[i];
    __syncthreads();
    for (int kb = 0; kb < nblk; kb++) {
        const int o = kb * CB;
        {
            const int row = tid >> 4, t = tid & 15;
            double acc = 0;
            for (int c = t; c < o; c += 16) acc += (double)A[(size_t)(o + row) * ld + c] * y[c];
            for (int off = 8; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
            __syncthreads();
            if (t == 0) y[o + row] -= acc;
        }
        __syncthreads();
        if (warp == 0) {
            for (int c = 0; c < CB; c++) {
                if (lane == 0) y[o + c] /= (double)A[(size_t)(o + c) * ld + o + c];
                __syncwarp();
                const double yc = y[o + c];
                for (int rr = c + 1 + lane; rr < CB; rr += 32) y[o + rr] -= (double)A[(size_t)(o + rr) * ld + o + c] * yc;
                __syncwarp();
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < Mp; i += blockDim.x) z[i] = 0;
    __syncthreads();
    for (int kb = nblk - 1; kb >= 0; kb--) {
        const int o = kb * CB, e = o + CB;
        {
            const int c = tid & 63, t = tid >> 6;
            double acc = 0;
            for (int rr = e + t; rr < Mp; rr += 16) acc += (double)A[(size_t)rr * ld + o + c] * z[rr];
            part[t][c] = acc;
        }
        __syncthreads();
        if (tid < CB) {
            double acc = 0;
            for (int t = 0; t < 16; t++) acc += part[t][tid];
            y[o + tid] -= acc;
        }
        __syncthreads();
        if (warp == 0) {
            for (int c = CB - 1; c >= 0; c--) {
                if (lane == 0) z[o + c] = y[o + c] / (double)A[(size_t)(o + c) * ld + o + c];
                __syncwarp();
                const double zc = z[o + c];
                for (int rr = lane; rr < c; rr += 32) y[o + rr] -= (double)A[(size_t)(o + c) * ld + o + rr] * zc;
                __syncwarp();
            }
        }
        __syncthreads();
    }
}

}  // namespace qlpix
