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

void sparseops_init_attributes()
{
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
// (nx + 2 (pnx/2)) (ny + 2 (pny/2)) doubles
void op_conv(const StaticData& sd, Work& w, int N_cap, bool transpose, const double* in, const double* scale_in,
             double* out, double* img, cudaStream_t st)
{
    const size_t npad = (size_t)(sd.nx + 2 * (sd.pnx / 2)) * (sd.ny + 2 * (sd.pny / 2));
    cudaMemsetAsync(img, 0, sizeof(double) * npad, st);
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
