// raytrace.cu -- FP64 ray shooting of the split image pixels.
//
// One thread per sub-pixel.  The sub-pixel centre and the lens equation are
// evaluated in QLens's operation order so that the source points agree with
// the reference to the last bit wherever the transcendental functions agree:
//   sub-pixel centre  (1-u0)*x_i + u0*x_{i+1}     set_nsplits, pixelgrid.cpp:10898-10938
//   beta = theta - sum_planes zfac_i alpha_i      QLens::deflection, lenscalc.cpp:81-113
//   per-lens shift / rotate / deflect / rotate    LensProfile::deflection, profile.cpp:1782-1805
// This file is compiled with --fmad=false: no multiply-add is contracted, the
// same as the reference on x86-64.
#include "qlpix_internal.h"
#include "lens_device.cuh"

namespace qlpix {

template <bool NFW>
__global__ void __launch_bounds__(256) k_raytrace(StaticData sd_, const EvalParams* __restrict__ ep,
                                                  double* __restrict__ spx, double* __restrict__ spy)
{
    const StaticData sd = eval_shape(sd_);
    // the lens model of this evaluation, staged in shared memory, and the
    // power-law series coefficients of each lens (the same bits the series
    // loop would compute; used only by core-free power laws)
    __shared__ __align__(16) LensModel lm;
    __shared__ double rho_tab[QLP_MAX_LENSES * SPLE_RHO_TAB];
    // the sub-pixel fractions u0 = (1 + 2 ii) / (2 ns) and 1 - u0, formed once
    // per CTA by the same expressions (the same bits): no FP64 divide per ray
    __shared__ double frac_u[SUBPIX_TAB], frac_1mu[SUBPIX_TAB];
    {
        const double* src = reinterpret_cast<const double*>(&ep->lm);
        double* dst = reinterpret_cast<double*>(&lm);
        for (int k = threadIdx.x; k < (int)(sizeof(LensModel) / sizeof(double)); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < lm.nlens * SPLE_RHO_TAB; e += blockDim.x) {
        const LensRec& L = lm.lens[e / SPLE_RHO_TAB];
        rho_tab[e] = (L.type == QLP_LENS_SPLE && L.kind == 2) ? sple_rho(L, e % SPLE_RHO_TAB + 1) : 0.0;
    }
    const int ns = sd.nsplit, nsub = sd.nsub;
    subpix_table(ns, frac_u, frac_1mu);
    __syncthreads();
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < sd.n_sub; t += gridDim.x * blockDim.x) {
        int m = t / nsub, k = t - m * nsub;
        int pix = sd.mpix[m];
        int i = pix / sd.ny, j = pix - i * sd.ny;
        int ii = k / ns, jj = k - ii * ns;
        double px, py;
        subpix_centre(sd, ns, ii, jj, i, j, frac_u, frac_1mu, px, py);
        double bx, by;
        find_sourcept<NFW>(lm, px, py, bx, by, rho_tab);
        spx[t] = bx;
        spy[t] = by;
    }
}

// nfw: the model has an NFW lens (selects the kernel with the quadrature);
// threads: CTA size (64, 128 or 256, from the context's schedule)
void launch_raytrace(const StaticData& sd, bool nfw, Work& w, int threads, cudaStream_t st)
{
    if (sd.n_sub == 0) return;
    if (threads != 64 && threads != 128) threads = 256;
    const int blocks = (sd.n_sub + threads - 1) / threads;
    if (nfw) k_raytrace<true><<<blocks, threads, 0, st>>>(sd, w.ep, w.spx, w.spy);
    else k_raytrace<false><<<blocks, threads, 0, st>>>(sd, w.ep, w.spx, w.spy);
    count_launches(1);
}

}  // namespace qlpix
