// outside.cu -- the outside-surface-brightness prior (QLens 'outside_sb_prior').
//
// After the inversion the reference re-makes the model image over the
// extended mask and penalises surface brightness it finds outside the mask
// (QLens::invert_image_surface_brightness_map, lens.cpp:13063-13158,
// Cartesian branch):
//   the grid switches to the extended mask (ImagePixelGrid::
//   activate_extended_mask, pixelgrid.cpp:10833-10852); pixels of the mask keep
//   their split, the others split emask_nsplit ways (set_nsplits 10898-10938);
//   their sub-pixels are ray-traced and mapped onto the source grid of the
//   inversion (assign_pixel_mappings 12777-12910); the amplitudes are the
//   inverted ones on the cells the inversion had active and zero elsewhere
//   (SourcePixel::update_surface_brightness 817-831); the model of a pixel is
//   its dense L row times those amplitudes, summed over cells in ascending
//   order (convert_Lmatrix_to_dense 13717-13747,
//   calculate_image_pixel_surface_brightness_dense 18268-18290); it is
//   PSF-convolved over the mapped extended-mask pixels
//   (PSF_convolution_pixel_vector, direct branch 14409-14493); then with the
//   peak over masked mapped pixels and t = max(noise_frac sigma, frac peak),
//   the largest |sb| >= t over mapped extended-mask pixels outside the mask
//   adds (1 + |(sb - t)/t|)^60 - 1 to -2 log(evidence).
// A neighbour in the extended mask that maps nowhere has pixel index -1 in
// the reference, which reads element -1 of its vector there; it counts as 0
// here.
//
// One thread per extended-mask sub-pixel for the rays and the cells, one per
// pixel for the model and the convolution, one CTA for the two maxima.  The
// file is compiled with --fmad=false, like the inversion's ray shooting and
// mapping, so the sub-pixel source points and L weights carry the same bits.
#include "qlpix_internal.h"
#include "lens_device.cuh"

namespace qlpix {

namespace {

// e such that eoff[e] <= t < eoff[e + 1]
__device__ __forceinline__ int owner(const int* __restrict__ eoff, int ne, int t)
{
    int lo = 0, hi = ne - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (eoff[mid] <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <bool NFW>
__global__ void __launch_bounds__(256) k_osb_rays(StaticData sd, const EvalParams* __restrict__ ep, OsbStatic os,
                                                  double* __restrict__ sp)
{
    __shared__ __align__(16) LensModel lm;
    __shared__ double rho_tab[QLP_MAX_LENSES * SPLE_RHO_TAB];
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
    __syncthreads();
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < os.nsub_e; t += gridDim.x * blockDim.x) {
        const int e = owner(os.eoff, os.ne, t);
        const int pix = os.epix[e];
        const int ns = os.inmask[pix] ? sd.nsplit : os.ens;
        const int k = t - os.eoff[e];
        const int i = pix / sd.ny, j = pix - i * sd.ny;
        const int ii = k / ns, jj = k - ii * ns;
        const double u0 = ((double)(1 + 2 * ii)) / (2 * ns);
        const double w0 = ((double)(1 + 2 * jj)) / (2 * ns);
        const double px = (1 - u0) * sd.xvals[i] + u0 * sd.xvals[i + 1];
        const double py = (1 - w0) * sd.yvals[j] + w0 * sd.yvals[j + 1];
        double bx, by;
        find_sourcept<NFW>(lm, px, py, bx, by, rho_tab);
        sp[2 * t] = bx;
        sp[2 * t + 1] = by;
    }
}

// containing cell, interpolation neighbours and weights, as the inversion's
// mapping (k_locate), with the pixel's own split in the weight
__global__ void __launch_bounds__(256) k_osb_locate(StaticData sd_, SrcOpts so_, OsbStatic os,
                                                    const double* __restrict__ sp, const double* __restrict__ cx,
                                                    const double* __restrict__ cy, const double* __restrict__ ccx,
                                                    const double* __restrict__ ccy, int* __restrict__ cell3,
                                                    double* __restrict__ w3)
{
    const SrcOpts so = eval_grid(so_, sd_);
    const int snx = so.snx, sny = so.sny;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < os.nsub_e; t += gridDim.x * blockDim.x) {
        const double px = sp[2 * t], py = sp[2 * t + 1];
        if (!(px >= cx[0] && px < cx[snx] && py >= cy[0] && py < cy[sny])) {
            cell3[3 * t] = -1; cell3[3 * t + 1] = -1; cell3[3 * t + 2] = -1;
            continue;
        }
        const int e = owner(os.eoff, os.ne, t);
        const int ns = os.inmask[os.epix[e]] ? sd_.nsplit : os.ens;
        const double weight = 1.0 / (ns * ns);
        int lo = 0, hi = snx - 1;
        while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (cx[mid] <= px) lo = mid; else hi = mid - 1; }
        const int ci = lo;
        lo = 0; hi = sny - 1;
        while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (cy[mid] <= py) lo = mid; else hi = mid - 1; }
        const int cj = lo;
        const int xn = ((px > ccx[ci] && ci < snx - 1) || ci == 0) ? ci + 1 : ci - 1;
        const int yn = ((py > ccy[cj] && cj < sny - 1) || cj == 0) ? cj + 1 : cj - 1;
        cell3[3 * t] = cj * snx + ci; cell3[3 * t + 1] = cj * snx + xn; cell3[3 * t + 2] = yn * snx + ci;
        const double p0x = ccx[ci], p0y = ccy[cj];
        const double p1x = ccx[xn], p1y = ccy[cj];
        const double p2x = ccx[ci], p2y = ccy[yn];
        const double d = (p0x - p1x) * (p1y - p2y) - (p1x - p2x) * (p0y - p1y);
        w3[3 * t]     = weight * (px * (p1y - p2y) + py * (p2x - p1x) + p1x * p2y - p1y * p2x) / d;
        w3[3 * t + 1] = weight * (px * (p2y - p0y) + py * (p0x - p2x) + p0y * p2x - p0x * p2y) / d;
        w3[3 * t + 2] = weight * (px * (p0y - p1y) + py * (p1x - p0x) + p0x * p1y - p0y * p1x) / d;
    }
}

// model of each extended-mask pixel: distinct cells in ascending order, each
// with its entries summed in L order, times the cell's amplitude
__global__ void __launch_bounds__(128) k_osb_model(OsbStatic os, const int* __restrict__ cell3,
                                                   const double* __restrict__ w3,
                                                   const int* __restrict__ active_index, const double* __restrict__ s,
                                                   double* __restrict__ model, int* __restrict__ act)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < os.ne; e += gridDim.x * blockDim.x) {
        const int t0 = os.eoff[e], t1 = os.eoff[e + 1];
        const int pix = os.epix[e];
        bool maps = false;
        for (int t = t0; t < t1; t++) maps |= (cell3[3 * t] >= 0);
        act[pix] = maps ? 1 : 0;
        if (!maps) { model[pix] = 0.0; continue; }
        double acc = 0.0;
        int last = -1;
        for (;;) {
            int next = 0x7fffffff;                  // smallest cell id above the last one
            for (int t = t0; t < t1; t++) {
                if (cell3[3 * t] < 0) continue;
                for (int u = 0; u < 3; u++) {
                    const int c = cell3[3 * t + u];
                    if (c > last && c < next) next = c;
                }
            }
            if (next == 0x7fffffff) break;
            double v = 0.0;
            for (int t = t0; t < t1; t++) {
                if (cell3[3 * t] < 0) continue;
                for (int u = 0; u < 3; u++) if (cell3[3 * t + u] == next) v += w3[3 * t + u];
            }
            const int a = active_index[next];
            acc += v * (a >= 0 ? s[a] : 0.0);
            last = next;
        }
        model[pix] = acc;
    }
}

__global__ void __launch_bounds__(128) k_osb_psf(StaticData sd, OsbStatic os, const double* __restrict__ model,
                                                 const int* __restrict__ act, double* __restrict__ sb)
{
    const int nx = sd.nx, ny = sd.ny, pnx = sd.pnx, pny = sd.pny, nxh = pnx / 2, nyh = pny / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < os.ne; e += gridDim.x * blockDim.x) {
        const int pix = os.epix[e];
        if (!act[pix]) { sb[pix] = 0.0; continue; }
        const int k = pix / ny, l = pix - k * ny;
        double v = 0.0;
        for (int pk = 0; pk < pnx; pk++) {
            const int ii = k + nxh - pk;
            if (ii < 0 || ii >= nx) continue;
            for (int pl = 0; pl < pny; pl++) {
                const int jj = l + nyh - pl;
                if (jj < 0 || jj >= ny) continue;
                const int q = ii * ny + jj;
                if (!os.emask[q] || !act[q]) continue;
                v += sd.psf[pk * pny + pl] * model[q];
            }
        }
        sb[pix] = v;
    }
}

__device__ __forceinline__ double block_max(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = -1e30;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) r = fmax(r, red[k]);
    return r;
}

__global__ void __launch_bounds__(1024) k_osb_penalty(OsbStatic os, const double* __restrict__ sb,
                                                      const int* __restrict__ act, EvalOut* out)
{
    __shared__ double red[32];
    double m = -1e30;
    for (int e = threadIdx.x; e < os.ne; e += blockDim.x) {
        const int pix = os.epix[e];
        if (os.inmask[pix] && act[pix]) m = fmax(m, sb[pix]);
    }
    const double max_sb = block_max(m, red);
    const double a = os.noise_frac * os.bg_noise, b = os.frac * max_sb;
    const double thr = (a > b) ? a : b;
    double x = -1e30;
    for (int e = threadIdx.x; e < os.ne; e += blockDim.x) {
        const int pix = os.epix[e];
        if (!os.inmask[pix] && act[pix] && fabs(sb[pix]) >= thr) x = fmax(x, fabs(sb[pix]));
    }
    const double max_ext = block_max(x, red);
    if (threadIdx.x == 0) {
        double pen = 0.0;
        if (max_ext > 0) pen = pow(1 + fabs((max_ext - thr) / thr), 60) - 1.0;
        out->osb_penalty = pen;
        if (out->status == 0) out->m2logev += pen;
    }
}

}  // namespace

void launch_outside_sb(const StaticData& sd_in, const SrcOpts& so, const OsbStatic& os, const OsbWork& ow, bool nfw,
                       Work& w, cudaStream_t st)
{
    StaticData sd = sd_in;
    if (os.ne == 0) return;
    const int tb = (os.nsub_e + 255) / 256;
    if (nfw) k_osb_rays<true><<<tb, 256, 0, st>>>(sd, w.ep, os, ow.sp);
    else k_osb_rays<false><<<tb, 256, 0, st>>>(sd, w.ep, os, ow.sp);
    k_osb_locate<<<tb, 256, 0, st>>>(sd, so, os, ow.sp, w.cx, w.cy, w.ccx, w.ccy, ow.cell3, ow.w3);
    const int pb = (os.ne + 127) / 128;
    k_osb_model<<<pb, 128, 0, st>>>(os, ow.cell3, ow.w3, w.active_index, w.s, ow.model, ow.act);
    k_osb_psf<<<pb, 128, 0, st>>>(sd, os, ow.model, ow.act, ow.sb);
    k_osb_penalty<<<1, 1024, 0, st>>>(os, ow.sb, ow.act, w.out);
    count_launches(5);
}

}  // namespace qlpix
