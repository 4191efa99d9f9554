// psf.cu -- PSF convolution of the lensing matrix into the dense L'.
//
// QLens::PSF_convolution_Lmatrix_dense, direct path (pixelgrid.cpp:14092-14176):
//   L'[p][s] = sum over PSF taps (k-major, then l) of psf[k][l] * Ldense[q][s],
//   q = the active pixel at (i_p + nx/2 - k, j_p + ny/2 - l).
// The reference multiplies every dense row; this kernel gathers only the
// merged nonzeros of each tapped row (about 3*nsub of M entries), adding them
// in the same tap order, so in FP64 every L' entry is the same sum of the same
// products in the same order (zero terms dropped).  One warp per output row
// accumulates in shared memory; taps are separated by __syncwarp so the
// per-entry order is the reference's.  Built with --fmad=false.
//
// The accumulator type is a template parameter; the plain path instantiates
// double (bit-exact rows).  The mixed path builds its TF32 operand column by
// column instead (k_psf_x, mixed.cu).
#include "qlpix_internal.h"

namespace qlpix {

#define PSF_G 8          // taps whose entries are loaded before they are applied

template <typename T>
__global__ void k_psf(StaticData sd, const GridState* __restrict__ gs, const int* __restrict__ rowpix,
                      const int* __restrict__ pixindex, const int* __restrict__ rowptr,
                      const int* __restrict__ cidx, const double* __restrict__ cval, const int* __restrict__ ccnt,
                      T* __restrict__ Lpsf, int ldL, int M_max)
{
    extern __shared__ __align__(16) unsigned char psf_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int nT = sd.pnx * sd.pny;
    const int Tpad = (nT + PSF_G - 1) / PSF_G * PSF_G;
    // per warp: M_max accumulators (T), Tpad psf values (T), Tpad (base, count)
    unsigned char* mine = psf_smem + (size_t)warp * (sizeof(T) * (M_max + Tpad) + sizeof(int2) * Tpad);
    T* acc = reinterpret_cast<T*>(mine);
    T* tpsf = acc + M_max;
    int2* tmeta = reinterpret_cast<int2*>(tpsf + Tpad);
    const int N = gs->N, M = gs->M;
    const int Mpad = (M + 63) & ~63;
    const int nxh = sd.pnx / 2, nyh = sd.pny / 2;
    for (int r = blockIdx.x * wpb + warp; r < N; r += gridDim.x * wpb) {
        for (int s = lane; s < Mpad; s += 32) acc[s] = T(0);
        const int pix = rowpix[r];
        const int k = pix / sd.ny, l = pix - k * sd.ny;
        // tap metadata, all loads independent
        for (int t = lane; t < Tpad; t += 32) {
            int base = 0, cnt = 0;
            T pv = 0;
            if (t < nT) {
                const int pk = t / sd.pny, pl = t - pk * sd.pny;
                const int ii = k + nxh - pk, jj = l + nyh - pl;
                if (ii >= 0 && ii < sd.nx && jj >= 0 && jj < sd.ny) {
                    const int q = pixindex[ii * sd.ny + jj];
                    if (q >= 0) { base = rowptr[q]; cnt = ccnt[q]; pv = (T)sd.psf[t]; }
                }
            }
            tmeta[t] = make_int2(base, cnt);
            tpsf[t] = pv;
        }
        __syncwarp();
        for (int t0 = 0; t0 < Tpad; t0 += PSF_G) {
            int si[PSF_G][2];
            T sv[PSF_G][2];
            #pragma unroll
            for (int g = 0; g < PSF_G; g++) {
                const int2 md = tmeta[t0 + g];
                const T pv = tpsf[t0 + g];
                #pragma unroll
                for (int j = 0; j < 2; j++) {
                    const int e = lane + 32 * j;
                    si[g][j] = -1;
                    sv[g][j] = 0;
                    if (e < md.y) { si[g][j] = cidx[md.x + e]; sv[g][j] = pv * (T)cval[md.x + e]; }
                }
            }
            #pragma unroll
            for (int g = 0; g < PSF_G; g++) {
                #pragma unroll
                for (int j = 0; j < 2; j++)
                    if (si[g][j] >= 0) acc[si[g][j]] = acc[si[g][j]] + sv[g][j];
                const int2 md = tmeta[t0 + g];
                if (md.y > 64) {   // rows with more than 64 merged entries: the rest in order
                    const T pv = tpsf[t0 + g];
                    for (int e = 64 + lane; e < md.y; e += 32) {
                        const int s = cidx[md.x + e];
                        acc[s] = acc[s] + pv * (T)cval[md.x + e];
                    }
                }
                __syncwarp();
            }
        }
        T* out = Lpsf + (size_t)r * ldL;
        for (int s = lane; s < Mpad; s += 32) out[s] = acc[s];
        __syncwarp();
    }
}

// Active row -> image pixel, the inverse of the compaction's pixindex.
__global__ void k_rowpix(StaticData sd_, const int* __restrict__ rowidx, int* __restrict__ rowpix)
{
    const StaticData sd = eval_shape(sd_);
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < sd.n_mask; m += gridDim.x * blockDim.x) {
        int r = rowidx[m];
        if (r >= 0) rowpix[r] = sd.mpix[m];
    }
}

void psf_init_attributes()
{
    cudaFuncSetAttribute(k_psf<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <typename T>
static size_t psf_bytes_per_warp(int M_max, int nT)
{
    const int Tpad = (nT + PSF_G - 1) / PSF_G * PSF_G;
    return sizeof(T) * ((size_t)M_max + Tpad) + sizeof(int2) * Tpad;
}

template <typename T>
static void launch_psf_t(const StaticData& sd, Work& w, T* out, int ld, int M_max, cudaStream_t st)
{
    if (sd.n_mask == 0) return;
    const int nT = sd.pnx * sd.pny;
    const size_t per_warp = psf_bytes_per_warp<T>(M_max, nT);
    int wpb = (int)((200 * 1024) / per_warp);
    if (wpb > 8) wpb = 8;
    if (wpb < 1) wpb = 1;
    int blocks = (sd.n_mask + wpb - 1) / wpb;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_psf<T><<<blocks, 32 * wpb, per_warp * wpb, st>>>(sd, w.gs, w.rowpix, w.pixindex, w.rowptr, w.cidx, w.cval,
                                                       w.ccnt, out, ld, M_max);
}

void launch_rowpix(const StaticData& sd, Work& w, cudaStream_t st)
{
    if (sd.n_mask == 0) return;
    k_rowpix<<<(sd.n_mask + 255) / 256, 256, 0, st>>>(sd, w.rowidx, w.rowpix);
    count_launches(1);
}

void launch_psf(const StaticData& sd, const SrcOpts& so, Work& w, int M_max, cudaStream_t st)
{
    (void)so;
    launch_psf_t<double>(sd, w, w.Lpsf, w.ldL, M_max, st);
    count_launches(1);
}

}  // namespace qlpix
