// sparseops.cu -- FP64 products with the PSF-convolved lensing matrix without
// forming it: L' = P L, where L is the pre-PSF lensing matrix (merged CSR
// rows, about 3*nsub entries per image pixel) and P the PSF convolution
// restricted to the active pixels (QLens::PSF_convolution_Lmatrix_dense,
// pixelgrid.cpp:14126-14168):
//     L' s       = P (L s)          k_Ls, k_conv
//     L'^T w     = L^T (P^T w)      k_convT, k_LTw_chunk + k_LTw_final
// Each costs a few million FP64 multiply-adds instead of N*M, so the
// mixed-precision path keeps its D = L'^T C^-1 d, refinement residuals and
// model image in FP64 at negligible cost.  All reductions run in a fixed
// order (no atomics), so results are reproducible run to run.
#include "qlpix_internal.h"

namespace qlpix {

// t[r] = sum_e cval[e] s[cidx[e]] over the merged row r (one thread per row)
__global__ void k_Ls(const GridState* __restrict__ gs, const int* __restrict__ rowptr, const int* __restrict__ cidx,
                     const double* __restrict__ cval, const int* __restrict__ ccnt, const double* __restrict__ s,
                     double* __restrict__ t)
{
    const int N = gs->N;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const int b = rowptr[r], n = ccnt[r];
        double acc = 0;
        for (int e = 0; e < n; e++) acc += cval[b + e] * s[cidx[b + e]];
        t[r] = acc;
    }
}

// out[p] = sum_taps psf[pk][pl] in[q], q at (i_p + nx/2 - pk, j_p + ny/2 - pl)   (P)
// out[q] = sum_taps psf[pk][pl] in[p], p at (i_q - nx/2 + pk, j_q - ny/2 + pl)   (P^T)
// One warp per output pixel, lanes over taps, fixed shuffle tree.
template <bool TRANSPOSE>
__global__ void __launch_bounds__(256) k_conv(StaticData sd, const GridState* __restrict__ gs,
                                              const int* __restrict__ rowpix, const int* __restrict__ pixindex,
                                              const double* __restrict__ in, const double* __restrict__ scale_in,
                                              double* __restrict__ out)
{
    const int N = gs->N;
    const int lane = threadIdx.x & 31;
    const int nT = sd.pnx * sd.pny, nxh = sd.pnx / 2, nyh = sd.pny / 2;
    for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < N; r += gridDim.x * (blockDim.x >> 5)) {
        const int pix = rowpix[r];
        const int k = pix / sd.ny, l = pix - k * sd.ny;
        double acc = 0;
        for (int t = lane; t < nT; t += 32) {
            const int pk = t / sd.pny, pl = t - pk * sd.pny;
            const int ii = TRANSPOSE ? k - nxh + pk : k + nxh - pk;
            const int jj = TRANSPOSE ? l - nyh + pl : l + nyh - pl;
            if (ii < 0 || ii >= sd.nx || jj < 0 || jj >= sd.ny) continue;
            const int q = pixindex[ii * sd.ny + jj];
            if (q < 0) continue;
            double v = in[q];
            if (scale_in) v *= scale_in[q];
            acc += sd.psf[t] * v;
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[r] = acc;
    }
}

// partial[chunk][s] = sum over the chunk's rows r (in order) of cval * w[r]
#define LTW_CHUNK 64
__global__ void __launch_bounds__(32) k_LTw_chunk(const GridState* __restrict__ gs, const int* __restrict__ rowptr,
                                                  const int* __restrict__ cidx, const double* __restrict__ cval,
                                                  const int* __restrict__ ccnt, const double* __restrict__ w,
                                                  double* __restrict__ part, int M_cap)
{
    extern __shared__ double acc_ltw[];
    const int N = gs->N, M = gs->M;
    const int r0 = blockIdx.x * LTW_CHUNK;
    if (r0 >= N) return;
    const int Mp = (M + 63) & ~63;
    for (int s = threadIdx.x; s < Mp; s += 32) acc_ltw[s] = 0;
    __syncwarp();
    const int r1 = min(r0 + LTW_CHUNK, N);
    for (int r = r0; r < r1; r++) {
        const int b = rowptr[r], n = ccnt[r];
        const double wr = w[r];
        for (int e = threadIdx.x; e < n; e += 32) {   // merged row: distinct columns
            const int s = cidx[b + e];
            acc_ltw[s] += cval[b + e] * wr;
        }
        __syncwarp();
    }
    double* dst = part + (size_t)blockIdx.x * M_cap;
    for (int s = threadIdx.x; s < Mp; s += 32) dst[s] = acc_ltw[s];
}

__global__ void k_LTw_final(const GridState* __restrict__ gs, const double* __restrict__ part, int M_cap,
                            double* __restrict__ out)
{
    const int N = gs->N, M = gs->M;
    const int Mp = (M + 63) & ~63;
    const int nch = (N + LTW_CHUNK - 1) / LTW_CHUNK;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < Mp; s += gridDim.x * blockDim.x) {
        double acc = 0;
        if (s < M)
            for (int c = 0; c < nch; c++) acc += part[(size_t)c * M_cap + s];
        out[s] = acc;
    }
}

void sparseops_init_attributes()
{
    cudaFuncSetAttribute(k_LTw_chunk, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
}

int ltw_chunks(int N_cap) { return (N_cap + LTW_CHUNK - 1) / LTW_CHUNK; }

// t = L s (image plane, active rows)
void op_Ls(Work& w, int N_cap, const double* s, double* t, cudaStream_t st)
{
    k_Ls<<<(N_cap + 255) / 256, 256, 0, st>>>(w.gs, w.rowptr, w.cidx, w.cval, w.ccnt, s, t);
    count_launches(1);
}

// out = P in, or P^T (scale .* in) when transpose
void op_conv(const StaticData& sd, Work& w, int N_cap, bool transpose, const double* in, const double* scale_in,
             double* out, cudaStream_t st)
{
    int blocks = (N_cap + 7) / 8;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (transpose)
        k_conv<true><<<blocks, 256, 0, st>>>(sd, w.gs, w.rowpix, w.pixindex, in, scale_in, out);
    else
        k_conv<false><<<blocks, 256, 0, st>>>(sd, w.gs, w.rowpix, w.pixindex, in, scale_in, out);
    count_launches(1);
}

// out = L^T v (source plane); part holds ltw_chunks(N_cap) x M_cap doubles
void op_LTw(Work& w, int N_cap, int M_cap, const double* v, double* part, double* out, cudaStream_t st)
{
    const int nch = ltw_chunks(N_cap);
    k_LTw_chunk<<<nch, 32, sizeof(double) * M_cap, st>>>(w.gs, w.rowptr, w.cidx, w.cval, w.ccnt, v, part, M_cap);
    k_LTw_final<<<(M_cap + 255) / 256, 256, 0, st>>>(w.gs, part, M_cap, out);
    count_launches(2);
}

}  // namespace qlpix
