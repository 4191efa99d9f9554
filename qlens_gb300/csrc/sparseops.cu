// sparseops.cu -- FP64 products with the PSF-convolved lensing matrix without
// forming it: L' = P L, where L is the pre-PSF lensing matrix (merged CSR
// rows, about 3*nsub entries per image pixel) and P the PSF convolution
// restricted to the active pixels (QLens::PSF_convolution_Lmatrix_dense,
// pixelgrid.cpp:14126-14168):
//     L' s       = P (L s)          k_Ls, k_conv
//     L'^T w     = L^T (P^T w)      k_convT, k_LTw_chunk + k_LTw_final
// Each costs a few million multiply-adds instead of N*M, so the
// mixed-precision path keeps its D = L'^T C^-1 d, refinement residuals and
// model image at FP64-level accuracy at small cost.  The convolutions run in
// double-float arithmetic on the FP32 pipe (k_conv_df: every value a pair of
// floats hi + lo, products split exactly with an FMA, sums compensated --
// about 2^-44 relative, against GB300's FP64 rate of 1/64 of FP32); PSFs too
// large for its shared-memory tiles take the FP64 kernel (k_conv).  All
// reductions run in a fixed order (no atomics), so results are reproducible
// run to run.
#include <algorithm>
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
// The input is first scattered (times scale_in, if any) into a dense image
// with a border of half a PSF on every side, zero at inactive pixels
// (k_scatter_img), so a tap is one load and one multiply-add with no table
// lookup or bounds check.  One warp per output pixel, lanes over taps in the
// same order as ever, fixed shuffle tree.
__global__ void k_scatter_img(StaticData sd, const GridState* __restrict__ gs, const int* __restrict__ rowpix,
                              const double* __restrict__ in, const double* __restrict__ scale_in,
                              double* __restrict__ img)
{
    const int N = gs->N;
    const int nxh = sd.pnx / 2, nyh = sd.pny / 2, nxp = sd.nx + 2 * nxh;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const int pix = rowpix[r];
        const int i = pix / sd.ny, j = pix - i * sd.ny;
        double v = in[r];
        if (scale_in) v *= scale_in[r];
        img[(size_t)(j + nyh) * nxp + i + nxh] = v;
    }
}

template <bool TRANSPOSE>
__global__ void __launch_bounds__(256) k_conv(StaticData sd, const GridState* __restrict__ gs,
                                              const int* __restrict__ rowpix, const double* __restrict__ img,
                                              double* __restrict__ out)
{
    // the taps' PSF values and offsets from the output pixel in the padded
    // image, tabulated once per CTA: a tap is then one shared load, one image
    // load and one multiply-add (no index arithmetic per tap)
    extern __shared__ __align__(16) unsigned char conv_smem[];
    const int N = gs->N;
    const int lane = threadIdx.x & 31;
    const int nT = sd.pnx * sd.pny, nxh = sd.pnx / 2, nyh = sd.pny / 2, nxp = sd.nx + 2 * nxh;
    double* tpsf = reinterpret_cast<double*>(conv_smem);
    int* toff = reinterpret_cast<int*>(tpsf + nT);
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        const int pk = t / sd.pny, pl = t - pk * sd.pny;
        tpsf[t] = sd.psf[t];
        toff[t] = TRANSPOSE ? pl * nxp + pk : (2 * nyh - pl) * nxp + (2 * nxh - pk);
    }
    __syncthreads();
    for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < N; r += gridDim.x * (blockDim.x >> 5)) {
        const int pix = rowpix[r];
        const int k = pix / sd.ny, l = pix - k * sd.ny;
        const double* base = img + (size_t)l * nxp + k;
        double acc = 0;
        for (int t = lane; t < nT; t += 32) acc += tpsf[t] * base[toff[t]];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[r] = acc;
    }
}

// The same products in double-float arithmetic over output tiles of
// CONV_TX x CONV_TY image pixels: the input is scattered as (hi, lo) float
// pairs into the dense padded image (k_scatter_df); a CTA stages its window
// (the tile plus the PSF's reach) and the PSF taps, split the same way, in
// shared memory, and each thread sums the taps of one output pixel.  A tap
// costs one broadcast load, one window load (consecutive lanes, consecutive
// pixels) and twelve FP32 operations:
//     h + e = v_hi t_hi exactly (e by an FMA),
//     (s_hi, err) = TwoSum(s_hi, h),
//     s_lo += (e + v_hi t_lo + v_lo t_hi) + err.
// Multiplies and adds are written with round-to-nearest intrinsics so that
// the compiler contracts none of them.  In window coordinates the tap (pk, pl)
// of P^T reads offset (pk, pl) and that of P reads (2 (pnx/2) - pk,
// 2 (pny/2) - pl), so one kernel serves both with its tap table reversed for
// P.  Tiles with no active pixel return at once; outputs go to the active
// rows through pixT (the padded image's row index, -1 outside the mask).
#define CONV_TX 32
#define CONV_TY 8

__global__ void k_scatter_df(StaticData sd, const GridState* __restrict__ gs, const int* __restrict__ rowpix,
                             const double* __restrict__ in, const double* __restrict__ scale_in,
                             float2* __restrict__ img)
{
    const int N = gs->N;
    const int nxh = sd.pnx / 2, nyh = sd.pny / 2, nxp = sd.nx + 2 * nxh;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const int pix = rowpix[r];
        const int i = pix / sd.ny, j = pix - i * sd.ny;
        double v = in[r];
        if (scale_in) v *= scale_in[r];
        const float hi = (float)v;
        img[(size_t)(j + nyh) * nxp + i + nxh] = make_float2(hi, (float)(v - (double)hi));
    }
}

__host__ __device__ __forceinline__ size_t conv_df_smem(int pnx, int pny)
{
    const size_t win = (size_t)(CONV_TX + 2 * (pnx / 2)) * (CONV_TY + 2 * (pny / 2));
    return sizeof(float2) * (win + (size_t)pnx * pny);
}

template <bool TRANSPOSE>
__global__ void __launch_bounds__(CONV_TX * CONV_TY) k_conv_df(StaticData sd, const int2* __restrict__ pixT,
                                                               const float2* __restrict__ img,
                                                               double* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char conv_smem[];
    const int pnx = sd.pnx, pny = sd.pny, nxh = pnx / 2, nyh = pny / 2;
    const int nxp = sd.nx + 2 * nxh, nyp = sd.ny + 2 * nyh;
    const int WX = CONV_TX + 2 * nxh, WY = CONV_TY + 2 * nyh;
    const int tx = threadIdx.x % CONV_TX, ty = threadIdx.x / CONV_TX;
    const int i0 = blockIdx.x * CONV_TX, j0 = blockIdx.y * CONV_TY;
    const int i = i0 + tx, j = j0 + ty;
    const int r = (i < sd.nx && j < sd.ny) ? pixT[(size_t)(j + nyh) * nxp + i + nxh].x : -1;
    if (!__syncthreads_or(r >= 0)) return;
    float2* win = reinterpret_cast<float2*>(conv_smem);
    float2* taps = win + (size_t)WX * WY;
    // window: padded-image columns i0 .. i0 + WX - 1, rows j0 .. j0 + WY - 1
    for (int e = threadIdx.x; e < WX * WY; e += blockDim.x) {
        const int wy = e / WX, wx = e - wy * WX;
        const int X = i0 + wx, Y = j0 + wy;
        win[e] = (X < nxp && Y < nyp) ? img[(size_t)Y * nxp + X] : make_float2(0.f, 0.f);
    }
    // taps in window order: entry (b, a) reads window offset (a0 + a, b0 + b)
    for (int e = threadIdx.x; e < pnx * pny; e += blockDim.x) {
        const int b = e / pnx, a = e - b * pnx;
        const int pk = TRANSPOSE ? a : pnx - 1 - a, pl = TRANSPOSE ? b : pny - 1 - b;
        const double t = sd.psf[pk * pny + pl];
        const float hi = (float)t;
        taps[e] = make_float2(hi, (float)(t - (double)hi));
    }
    __syncthreads();
    if (r < 0) return;
    const int a0 = TRANSPOSE ? 0 : 2 * nxh - pnx + 1, b0 = TRANSPOSE ? 0 : 2 * nyh - pny + 1;
    float sh = 0.f, sl = 0.f;
    const float2* tp = taps;
    for (int b = 0; b < pny; b++) {
        const float2* wr = win + (size_t)(ty + b0 + b) * WX + tx + a0;
        #pragma unroll 4
        for (int a = 0; a < pnx; a++) {
            const float2 T = tp[a];
            const float2 v = wr[a];
            const float h = __fmul_rn(v.x, T.x);
            const float e = __fmaf_rn(v.x, T.x, -h);
            const float s = __fadd_rn(sh, h);
            const float bb = __fsub_rn(s, sh);
            const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(h, bb));
            sh = s;
            sl = __fadd_rn(sl, __fadd_rn(__fmaf_rn(v.y, T.x, __fmaf_rn(v.x, T.y, e)), err));
        }
        tp += pnx;
    }
    out[r] = (double)sh + (double)sl;
}

void sparseops_init_attributes()
{
    cudaFuncSetAttribute(k_conv_df<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_conv_df<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_conv<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_conv<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

// t = L s (image plane, active rows)
void op_Ls(Work& w, int N_cap, const double* s, double* t, cudaStream_t st)
{
    k_Ls<<<(N_cap + 255) / 256, 256, 0, st>>>(w.gs, w.rowptr, w.cidx, w.cval, w.ccnt, s, t);
    count_launches(1);
}

// out = P in, or P^T (scale .* in) when transpose; img: scratch of
// (nx + 2 (pnx/2)) (ny + 2 (pny/2)) doubles; pixT: the active row of every
// padded-image pixel (-1 elsewhere)
void op_conv(const StaticData& sd, Work& w, int N_cap, bool transpose, const double* in, const double* scale_in,
             double* out, double* img, const int2* pixT, cudaStream_t st)
{
    const size_t npad = (size_t)(sd.nx + 2 * (sd.pnx / 2)) * (sd.ny + 2 * (sd.pny / 2));
    cudaMemsetAsync(img, 0, sizeof(double) * npad, st);
    const size_t smem_df = conv_df_smem(sd.pnx, sd.pny);
    if (smem_df <= 160 * 1024) {
        float2* img2 = reinterpret_cast<float2*>(img);
        k_scatter_df<<<std::max(1, std::min((N_cap + 255) / 256, 152 * 8)), 256, 0, st>>>(sd, w.gs, w.rowpix, in,
                                                                                         scale_in, img2);
        const dim3 grid((sd.nx + CONV_TX - 1) / CONV_TX, (sd.ny + CONV_TY - 1) / CONV_TY);
        if (transpose)
            k_conv_df<true><<<grid, CONV_TX * CONV_TY, smem_df, st>>>(sd, pixT, img2, out);
        else
            k_conv_df<false><<<grid, CONV_TX * CONV_TY, smem_df, st>>>(sd, pixT, img2, out);
        count_launches(2);
        return;
    }
    k_scatter_img<<<std::max(1, std::min((N_cap + 255) / 256, 152 * 8)), 256, 0, st>>>(sd, w.gs, w.rowpix, in,
                                                                                     scale_in, img);
    // the tap tables are staged once per CTA: CTAs that loop over several
    // rows amortise them (eight CTAs per SM resident)
    const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)sd.pnx * sd.pny;
    int blocks = (N_cap + 7) / 8;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (transpose)
        k_conv<true><<<std::max(blocks, 1), 256, smem, st>>>(sd, w.gs, w.rowpix, img, out);
    else
        k_conv<false><<<std::max(blocks, 1), 256, smem, st>>>(sd, w.gs, w.rowpix, img, out);
    count_launches(2);
}


}  // namespace qlpix
