// psf.cu -- PSF convolution of the lensing matrix into the dense L'.
//
// QLens::PSF_convolution_Lmatrix_dense, direct path (pixelgrid.cpp:14092-14176):
//   L'[p][s] = sum over PSF taps (k-major, then l) of psf[k][l] * Ldense[q][s],
//   q = the active pixel at (i_p + nx/2 - k, j_p + ny/2 - l).
// The reference multiplies every dense row; this kernel gathers only the
// merged nonzeros of each tapped row (about 3*nsub of M entries), adding them
// in the same tap order, so every L' entry is the same sum of the same
// products in the same order (zero terms dropped).  One warp per output row
// accumulates in shared memory; taps are separated by __syncwarp so the
// per-entry order is the reference's.  Built with --fmad=false.
#include "qlpix_internal.h"

namespace qlpix {

__global__ void k_psf(StaticData sd, const GridState* __restrict__ gs, const int* __restrict__ rowpix,
                      const int* __restrict__ pixindex, const int* __restrict__ rowptr,
                      const int* __restrict__ cidx, const double* __restrict__ cval, const int* __restrict__ ccnt,
                      double* __restrict__ Lpsf, int ldL, int M_max)
{
    extern __shared__ double acc_all[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    double* acc = acc_all + (size_t)warp * M_max;
    const int N = gs->N, M = gs->M;
    const int Mpad = (M + 63) & ~63;
    const int nxh = sd.pnx / 2, nyh = sd.pny / 2;
    for (int r = blockIdx.x * wpb + warp; r < N; r += gridDim.x * wpb) {
        for (int s = lane; s < Mpad; s += 32) acc[s] = 0.0;
        __syncwarp();
        const int pix = rowpix[r];
        const int k = pix / sd.ny, l = pix - k * sd.ny;
        for (int pk = 0; pk < sd.pnx; pk++) {
            const int ii = k + nxh - pk;
            if (ii < 0 || ii >= sd.nx) continue;
            for (int pl = 0; pl < sd.pny; pl++) {
                const int jj = l + nyh - pl;
                if (jj < 0 || jj >= sd.ny) continue;
                const int q = pixindex[ii * sd.ny + jj];
                if (q < 0) continue;
                const double pv = sd.psf[pk * sd.pny + pl];
                const int base = rowptr[q], cnt = ccnt[q];
                for (int e = lane; e < cnt; e += 32) {
                    const int s = cidx[base + e];
                    acc[s] = acc[s] + pv * cval[base + e];
                }
                __syncwarp();
            }
        }
        double* out = Lpsf + (size_t)r * ldL;
        for (int s = lane; s < Mpad; s += 32) out[s] = acc[s];
        __syncwarp();
    }
}

// Active row -> image pixel, the inverse of the compaction's pixindex.
__global__ void k_rowpix(StaticData sd, const int* __restrict__ rowidx, int* __restrict__ rowpix)
{
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < sd.n_mask; m += gridDim.x * blockDim.x) {
        int r = rowidx[m];
        if (r >= 0) rowpix[r] = sd.mpix[m];
    }
}

void psf_init_attributes()
{
    cudaFuncSetAttribute(k_psf, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

int psf_warps_per_block(int M_max)
{
    size_t per_warp = sizeof(double) * (size_t)M_max;
    int w = (int)((200 * 1024) / per_warp);
    if (w > 8) w = 8;
    if (w < 1) w = 1;
    return w;
}

void launch_psf(const StaticData& sd, const SrcOpts& so, Work& w, int M_max, cudaStream_t st)
{
    (void)so;
    if (sd.n_mask == 0) return;
    k_rowpix<<<(sd.n_mask + 255) / 256, 256, 0, st>>>(sd, w.rowidx, w.rowpix);
    const int wpb = psf_warps_per_block(M_max);
    const size_t smem = sizeof(double) * (size_t)M_max * wpb;
    int blocks = (sd.n_mask + wpb - 1) / wpb;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_psf<<<blocks, 32 * wpb, smem, st>>>(sd, w.gs, w.rowpix, w.pixindex, w.rowptr, w.cidx, w.cval, w.ccnt, w.Lpsf,
                                          w.ldL, M_max);
    count_launches(2);
}

}  // namespace qlpix
