// sur_exact.cu -- the exact re-shooting of surrogate rays near the source
// grid's decisions.  Compiled with --fmad=false like raytrace.cu, so that a
// ray traced here gets the plain path's bits (the surrogate ray shooting in
// surrogate.cu is compiled with contraction: its results are bounded by its
// error estimate, not bit-identical).
#include <algorithm>
#include "qlpix_ctx.h"
#include "lens_device.cuh"

namespace qlpix {

// ---------------------------------------------------------------------------
// Exact rays where the grid decides.  QLens's likelihood is not continuous in
// the source points: which cells a sub-pixel maps to changes at cell edges
// and at the lines through cell centres (SourcePixelGrid::
// assign_source_mapping_flags_interpolate, pixelgrid.cpp:2343-2432), and
// the grid itself is laid out from the extremes of the per-pixel mean source
// points (find_optimal_sourcegrid, pixelgrid.cpp:10998-11080).  A ray moved
// by the surrogate's error across such a line changes L by a finite step.
// So every ray whose error bound (sur_eps) reaches a decision is traced again
// with the plain path's own code (find_sourcept with the quadrature,
// lens_device.cuh, compiled without contraction), which gives the plain
// path's bits:
//   k_sur_exact_extremes  after a first grid: lists the rays of every pixel
//                         whose mean could be an extreme (within twice the
//                         largest bound); once they are traced the grid is
//                         laid out again and its extremes are the plain path's;
//   k_sur_exact_cells     after the final grid: lists every ray within its
//                         bound of a cell edge, a centre line or the grid's
//                         border;
//   k_sur_exact_trace     traces the listed rays, one warp per ray spread over
//                         the GPU (the NFW quadrature's nodes over the lanes).
// Afterwards the cells of every sub-pixel, the active set and L's sparsity
// are the plain path's; only the weights move, continuously.
// ---------------------------------------------------------------------------
// Ray t traced by the whole warp (all 32 lanes, converged, the same t): the
// NFW quadrature's nodes are spread over the lanes (nfw_integrals_warp, the
// same bits), every lane holds the result, lane 0 stores it.  wbuf: the
// warp's 2 QLP_PAT_N doubles of shared memory.
#define SUR_EXACT_THREADS 256
#define SUR_EXACT_WBUF (2 * QLP_PAT_N)
__device__ __forceinline__ void sur_exact_ray(const StaticData& sd, const LensModel& lm, const double* rho_tab,
                                              int t, double* spx, double* spy, double* wbuf)
{
    const int ns = sd.nsplit, nsub = sd.nsub;
    const int m = t / nsub, k = t - m * nsub;
    const int pix = sd.mpix[m];
    const int i = pix / sd.ny, j = pix - i * sd.ny;
    const int ii = k / ns, jj = k - ii * ns;
    const double u0 = ((double)(1 + 2 * ii)) / (2 * ns);
    const double w0 = ((double)(1 + 2 * jj)) / (2 * ns);
    const double px = (1 - u0) * sd.xvals[i] + u0 * sd.xvals[i + 1];
    const double py = (1 - w0) * sd.yvals[j] + w0 * sd.yvals[j + 1];
    double bx, by;
    find_sourcept<true>(lm, px, py, bx, by, rho_tab, wbuf);
    if ((threadIdx.x & 31) == 0) {
        spx[t] = bx;
        spy[t] = by;
    }
}

// the lens model and the power-law coefficients in shared memory, as k_raytrace stages them
__device__ __forceinline__ void sur_stage_model(const EvalParams* __restrict__ ep, LensModel& lm, double* rho_tab)
{
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
}

__global__ void __launch_bounds__(256) k_sur_exact_extremes(StaticData sd_, SrcOpts so,
                                                            const double* __restrict__ spx,
                                                            const double* __restrict__ spy,
                                                            const float* __restrict__ sur_eps, const GridState* gs,
                                                            double eps_g, int* __restrict__ n_exact,
                                                            int* __restrict__ xlist, int* __restrict__ xcount)
{
    const StaticData sd = eval_shape(sd_);
    const int nsub = sd.nsub;
    const bool use_nt = so.noise_threshold > 0;
    const double e0 = gs->ext[0], e1 = gs->ext[1], e2 = gs->ext[2], e3 = gs->ext[3];
    int cnt = 0;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < sd.n_mask; m += gridDim.x * blockDim.x) {
        if (use_nt) {
            const int pix = sd.mpix[m];
            if (sd.data[pix] <= so.noise_threshold * sqrt(1.0 / sd.covinv[pix])) continue;
        }
        double xs = 0, ys = 0;
        float emax = 0.f;
        for (int k = 0; k < nsub; k++) {
            xs += spx[m * nsub + k];
            ys += spy[m * nsub + k];
            emax = fmaxf(emax, sur_eps[m * nsub + k]);
        }
        if (emax == 0.f) continue;
        // the mean as k_grid_partial forms it (a multiply by the exact
        // reciprocal for a power-of-two count: the same quotient)
        if ((nsub & (nsub - 1)) == 0) { const double inv = 1.0 / nsub; xs *= inv; ys *= inv; }
        else { xs /= nsub; ys /= nsub; }
        const double tol = 2.0 * eps_g;
        const bool near = fabs(xs - e0) <= tol || fabs(xs - e1) <= tol || fabs(ys - e2) <= tol || fabs(ys - e3) <= tol;
        if (!near) continue;
        const int at = atomicAdd(xcount, nsub);                          // traced by k_sur_exact_trace
        for (int k = 0; k < nsub; k++) xlist[at + k] = m * nsub + k;
        cnt += nsub;
    }
    if (cnt) atomicAdd(n_exact, cnt);
}

// the listed rays, one warp each (grid-stride over the list)
__global__ void __launch_bounds__(SUR_EXACT_THREADS) k_sur_exact_trace(StaticData sd_,
                                                                       const EvalParams* __restrict__ ep,
                                                                       double* __restrict__ spx,
                                                                       double* __restrict__ spy,
                                                                       float* __restrict__ sur_eps,
                                                                       const int* __restrict__ xlist,
                                                                       const int* __restrict__ xcount)
{
    extern __shared__ double dsm[];
    const StaticData sd = eval_shape(sd_);
    __shared__ __align__(16) LensModel lm;
    __shared__ double rho_tab[QLP_MAX_LENSES * SPLE_RHO_TAB];
    const int n = *xcount;
    if ((int)blockIdx.x * (SUR_EXACT_THREADS / 32) >= n) return;
    sur_stage_model(ep, lm, rho_tab);
    const int lane = threadIdx.x & 31;
    double* wbuf = dsm + (threadIdx.x >> 5) * SUR_EXACT_WBUF;
    for (int e = blockIdx.x * (SUR_EXACT_THREADS / 32) + (threadIdx.x >> 5); e < n;
         e += gridDim.x * (SUR_EXACT_THREADS / 32)) {
        const int t = xlist[e];
        sur_exact_ray(sd, lm, rho_tab, t, spx, spy, wbuf);
        if (lane == 0) sur_eps[t] = 0.f;
    }
}

// distance from v to the decision lines of one axis: the grid's border when
// outside it, else the edges of its cell and the line through its centre
__device__ __forceinline__ double sur_axis_margin(double v, const double* c, const double* cc, int n)
{
    if (!(v >= c[0] && v < c[n])) return fmin(fabs(v - c[0]), fabs(v - c[n]));
    int lo = 0, hi = n - 1;
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (c[mid] <= v) lo = mid; else hi = mid - 1; }
    return fmin(fmin(v - c[lo], c[lo + 1] - v), fabs(v - cc[lo]));
}

// The same distance in FP32, for a prefilter: with v and the grid lines
// rounded to float, it is within fp32_slack of the FP64 distance (a float
// search that lands in a neighbouring cell does so only within rounding of
// the line between them, where both distances are below the slack).
__device__ __forceinline__ float sur_axis_margin_f(float v, const float* c, const float* cc, int n)
{
    if (!(v >= c[0] && v < c[n])) return fminf(fabsf(v - c[0]), fabsf(v - c[n]));
    int lo = 0, hi = n - 1;
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (c[mid] <= v) lo = mid; else hi = mid - 1; }
    return fminf(fminf(v - c[lo], c[lo + 1] - v), fabsf(v - cc[lo]));
}

__global__ void __launch_bounds__(256) k_sur_exact_cells(StaticData sd_, SrcOpts so_,
                                                         const double* __restrict__ spx, const double* __restrict__ spy,
                                                         float* __restrict__ sur_eps, const double* __restrict__ cx_g,
                                                         const double* __restrict__ cy_g,
                                                         const double* __restrict__ ccx_g,
                                                         const double* __restrict__ ccy_g, int* __restrict__ n_exact,
                                                         int* __restrict__ xlist, int* __restrict__ xcount)
{
    extern __shared__ double dsm[];
    const StaticData sd = eval_shape(sd_);
    const SrcOpts so = eval_grid(so_, sd_);
    __shared__ float cmax_sh;
    const int snx = so.snx, sny = so.sny;
    double* cx = dsm;
    double* cy = cx + snx + 1;
    double* ccx = cy + sny + 1;
    double* ccy = ccx + snx;
    float* cxf = reinterpret_cast<float*>(ccy + sny);
    float* cyf = cxf + snx + 1;
    float* ccxf = cyf + sny + 1;
    float* ccyf = ccxf + snx;
    if (threadIdx.x == 0) cmax_sh = 0.f;
    for (int i = threadIdx.x; i <= snx; i += blockDim.x) { cx[i] = cx_g[i]; cxf[i] = (float)cx[i]; }
    for (int j = threadIdx.x; j <= sny; j += blockDim.x) { cy[j] = cy_g[j]; cyf[j] = (float)cy[j]; }
    for (int i = threadIdx.x; i < snx; i += blockDim.x) { ccx[i] = ccx_g[i]; ccxf[i] = (float)ccx[i]; }
    for (int j = threadIdx.x; j < sny; j += blockDim.x) { ccy[j] = ccy_g[j]; ccyf[j] = (float)ccy[j]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float c = fmaxf(fmaxf(fabsf(cxf[0]), fabsf(cxf[snx])), fmaxf(fabsf(cyf[0]), fabsf(cyf[sny])));
        cmax_sh = c;
    }
    __syncthreads();
    const float cmax = cmax_sh;
    int cnt = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < sd.n_sub; t += gridDim.x * blockDim.x) {
        bool need = false;
        const float ef = sur_eps[t];
        if (ef != 0.f) {
            // FP32 prefilter: the float distances differ from the FP64 ones by
            // less than a few ulps of the coordinates' magnitude, so a ray clear
            // of every line by its bound plus that slack is clear in FP64 too
            // (a NaN fails the test and goes on to the FP64 check)
            const double vx = spx[t], vy = spy[t];
            const float fx = (float)vx, fy = (float)vy;
            const float dxf = sur_axis_margin_f(fx, cxf, ccxf, snx), dyf = sur_axis_margin_f(fy, cyf, ccyf, sny);
            const float lim = ef + 1e-6f * (fmaxf(fabsf(fx), fabsf(fy)) + cmax) + 1e-30f;
            if (!(dxf > lim && dyf > lim)) {
                const double e = ef;
                const double dx = sur_axis_margin(vx, cx, ccx, snx), dy = sur_axis_margin(vy, cy, ccy, sny);
                need = dx <= e || dy <= e || dx != dx || dy != dy;
            }
        }
        if (need) {
            xlist[atomicAdd(xcount, 1)] = t;                   // traced by k_sur_exact_trace
            cnt++;
        }
    }
    if (cnt) atomicAdd(n_exact, cnt);
}

void sur_exact_init_attributes()
{
    const int wb = (int)(sizeof(double) * (SUR_EXACT_THREADS / 32) * SUR_EXACT_WBUF);
    cudaFuncSetAttribute(k_sur_exact_trace, cudaFuncAttributeMaxDynamicSharedMemorySize, wb);
}

int launch_surrogate_exact(const StaticData& sd, const SrcOpts& so, Work& w, double eps_g, int step,
                           cudaStream_t st)
{
    if (sd.n_sub == 0) return QLP_OK;
    if (step == 0 && !so.auto_grid) return QLP_OK;
    cudaMemsetAsync(w.xcount, 0, sizeof(int), st);
    if (step == 0) {
        const int blocks = std::max(1, std::min((sd.n_mask + 255) / 256, 152 * 8));
        k_sur_exact_extremes<<<blocks, 256, 0, st>>>(sd, so, w.spx, w.spy, w.sur_eps, w.gs, eps_g,
                                                      &w.out->n_exact, w.xlist, w.xcount);
    } else {
        const size_t smem = (sizeof(double) + sizeof(float)) * (2 * (so.snx + so.sny) + 2);
        const int blocks = std::max(1, std::min((sd.n_sub + 255) / 256, 152 * 8));
        k_sur_exact_cells<<<blocks, 256, smem, st>>>(sd, so, w.spx, w.spy, w.sur_eps, w.cx, w.cy, w.ccx, w.ccy,
                                                     &w.out->n_exact, w.xlist, w.xcount);
    }
    // the listed rays: 2 CTAs per SM of 8 warps, a warp per ray
    const size_t wb = sizeof(double) * (SUR_EXACT_THREADS / 32) * SUR_EXACT_WBUF;
    k_sur_exact_trace<<<152 * 2, SUR_EXACT_THREADS, wb, st>>>(sd, w.ep, w.spx, w.spy, w.sur_eps, w.xlist,
                                                              w.xcount);
    count_launches(2);
    return QLP_OK;
}

}  // namespace qlpix
