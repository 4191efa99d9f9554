// mapping.cu -- source grid, sub-pixel -> source-cell mapping, active-set
// compaction and the pre-PSF lensing matrix L.
//
// Compiled with --fmad=false: the grid corners, cell centres and the 3-point
// interpolation weights are evaluated in QLens's operation order, so for equal
// source points the cell indices and L weights equal the reference's bit for
// bit.
#include "qlpix_internal.h"
#include <cfloat>
#include <algorithm>

namespace qlpix {

// ---------------------------------------------------------------------------
// Source-grid bounds and cells.
//   ImagePixelGrid::find_optimal_sourcegrid       pixelgrid.cpp:10998-11080
//   srcgrid_size_scale widening                    lens.cpp:12459-12470
//   SourcePixelGrid::create_pixel_grid            pixelgrid.cpp:401-472 (x += xstep accumulation)
//   SourcePixel ctor: centre = mean of 4 corners   pixelgrid.cpp:761-783
// k_grid_partial: per block, the min/max of the per-pixel mean source points
// (each mean summed in sub-pixel order) over a share of the masked pixels;
// k_grid: one block combines the partials (min and max are exact in any
// order) and thread 0 lays out the corners sequentially.  The clamp to the
// sourcegrid limits is order independent: bound = (extreme beyond limit) ?
// limit : extreme.
// ---------------------------------------------------------------------------
#define GRID_PARTS 1024
__global__ void __launch_bounds__(256) k_grid_partial(StaticData sd_, SrcOpts so, const double* __restrict__ spx,
                                                      const double* __restrict__ spy, double* __restrict__ part,
                                                      int* __restrict__ part_cnt)
{
    const StaticData sd = eval_shape(sd_);
    __shared__ double red[4][8];
    __shared__ int cnt_s[8];
    double xmn = DBL_MAX, xmx = -DBL_MAX, ymn = DBL_MAX, ymx = -DBL_MAX;
    int cnt = 0;
    if (so.auto_grid) {
        const int nsub = sd.nsub;
        const bool use_nt = so.noise_threshold > 0;
        // a power-of-two count divides as a multiply by its exact reciprocal
        // (the same correctly rounded quotient, without the FP64 divide)
        const bool pow2 = (nsub & (nsub - 1)) == 0;
        const double inv_nsub = 1.0 / nsub;
        for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < sd.n_mask; m += gridDim.x * blockDim.x) {
            if (use_nt) {
                int pix = sd.mpix[m];
                double noise = sqrt(1.0 / sd.covinv[pix]);
                if (sd.data[pix] <= so.noise_threshold * noise) continue;
            }
            double xs = 0, ys = 0;
            for (int k = 0; k < nsub; k++) { xs += spx[m * nsub + k]; ys += spy[m * nsub + k]; }
            if (pow2) { xs *= inv_nsub; ys *= inv_nsub; } else { xs /= nsub; ys /= nsub; }
            // NaN means are skipped, like the reference's failed comparisons
            if (xs == xs) { xmn = fmin(xmn, xs); xmx = fmax(xmx, xs); }
            if (ys == ys) { ymn = fmin(ymn, ys); ymx = fmax(ymx, ys); }
            cnt++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        xmn = fmin(xmn, __shfl_xor_sync(0xffffffffu, xmn, o));
        xmx = fmax(xmx, __shfl_xor_sync(0xffffffffu, xmx, o));
        ymn = fmin(ymn, __shfl_xor_sync(0xffffffffu, ymn, o));
        ymx = fmax(ymx, __shfl_xor_sync(0xffffffffu, ymx, o));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) { red[0][warp] = xmn; red[1][warp] = xmx; red[2][warp] = ymn; red[3][warp] = ymx; cnt_s[warp] = cnt; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; k++) {
            xmn = fmin(xmn, red[0][k]); xmx = fmax(xmx, red[1][k]);
            ymn = fmin(ymn, red[2][k]); ymx = fmax(ymx, red[3][k]);
            cnt += cnt_s[k];
        }
        part[4 * blockIdx.x] = xmn; part[4 * blockIdx.x + 1] = xmx;
        part[4 * blockIdx.x + 2] = ymn; part[4 * blockIdx.x + 3] = ymx;
        part_cnt[blockIdx.x] = cnt;
    }
}

__global__ void __launch_bounds__(1024) k_grid(StaticData sd_, SrcOpts so_, int nparts,
                                               const double* __restrict__ part, double* cx, double* cy,
                                               double* ccx, double* ccy, GridState* gs)
{
    const SrcOpts so = eval_grid(so_, sd_);
    __shared__ double red[4][32];
    double xmn = DBL_MAX, xmx = -DBL_MAX, ymn = DBL_MAX, ymx = -DBL_MAX;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
        xmn = fmin(xmn, part[4 * k]); xmx = fmax(xmx, part[4 * k + 1]);
        ymn = fmin(ymn, part[4 * k + 2]); ymx = fmax(ymx, part[4 * k + 3]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        xmn = fmin(xmn, __shfl_xor_sync(0xffffffffu, xmn, o));
        xmx = fmax(xmx, __shfl_xor_sync(0xffffffffu, xmx, o));
        ymn = fmin(ymn, __shfl_xor_sync(0xffffffffu, ymn, o));
        ymx = fmax(ymx, __shfl_xor_sync(0xffffffffu, ymx, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) { red[0][warp] = xmn; red[1][warp] = xmx; red[2][warp] = ymn; red[3][warp] = ymx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; k++) {
            xmn = fmin(xmn, red[0][k]); xmx = fmax(xmx, red[1][k]);
            ymn = fmin(ymn, red[2][k]); ymx = fmax(ymx, red[3][k]);
        }
        double gxmin, gxmax, gymin, gymax;
        gs->ext[0] = xmn; gs->ext[1] = xmx; gs->ext[2] = ymn; gs->ext[3] = ymx;
        if (so.auto_grid) {
            gxmin = 1e30; gxmax = -1e30; gymin = 1e30; gymax = -1e30;
            if (xmn != DBL_MAX) gxmin = (xmn > so.lxmin) ? xmn : so.lxmin;
            if (xmx != -DBL_MAX) gxmax = (xmx < so.lxmax) ? xmx : so.lxmax;
            if (ymn != DBL_MAX) gymin = (ymn > so.lymin) ? ymn : so.lymin;
            if (ymx != -DBL_MAX) gymax = (ymx < so.lymax) ? ymx : so.lymax;
            double xw = 0.1 * (gxmax - gxmin), yw = 0.1 * (gymax - gymin);
            gxmin -= xw / 2; gxmax += xw / 2; gymin -= yw / 2; gymax += yw / 2;
            if (so.size_scale != 0) {
                double xwa = so.size_scale * (gxmax - gxmin), ywa = so.size_scale * (gymax - gymin);
                double xc = (gxmax + gxmin) / 2, yc = (gymax + gymin) / 2;
                gxmin = xc - xwa / 2; gxmax = xc + xwa / 2; gymin = yc - ywa / 2; gymax = yc + ywa / 2;
            }
        } else {
            gxmin = so.xmin; gxmax = so.xmax; gymin = so.ymin; gymax = so.ymax;
        }
        gs->xmin = gxmin; gs->xmax = gxmax; gs->ymin = gymin; gs->ymax = gymax;
        gs->snx = so.snx; gs->sny = so.sny;
        gs->M = 0; gs->N = 0; gs->nnz = 0; gs->status = 0; gs->not_spd_F = 0; gs->not_spd_R = 0;
        double xstep = (gxmax - gxmin) / so.snx, ystep = (gymax - gymin) / so.sny;
        double x = gxmin;
        for (int i = 0; i <= so.snx; i++, x += xstep) cx[i] = x;
        double y = gymin;
        for (int j = 0; j <= so.sny; j++, y += ystep) cy[j] = y;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < so.snx; i += blockDim.x) ccx[i] = (cx[i] + cx[i] + cx[i + 1] + cx[i + 1]) / 4.0;
    for (int j = threadIdx.x; j < so.sny; j += blockDim.x) ccy[j] = (cy[j] + cy[j + 1] + cy[j] + cy[j + 1]) / 4.0;
}

void launch_grid(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st)
{
    const int nparts = std::max(1, std::min(GRID_PARTS, (sd.n_mask + 255) / 256));
    k_grid_partial<<<nparts, 256, 0, st>>>(sd, so, w.spx, w.spy, w.gpart, w.gpart_cnt);
    k_grid<<<1, 1024, 0, st>>>(sd, so, nparts, w.gpart, w.cx, w.cy, w.ccx, w.ccy, w.gs);
    count_launches(2);
}

// ---------------------------------------------------------------------------
// Per sub-pixel: containing cell, x/y interpolation neighbours and the three
// barycentric weights.
//   SourcePixelGrid::bisection_search_interpolate      pixelgrid.cpp:2291-2341
//   assign_source_mapping_flags_interpolate            pixelgrid.cpp:2343-2432
//   calculate_Lmatrix_interpolate (weights)            pixelgrid.cpp:2501-2527
// The reference's quadrant bisection over half-open rectangles selects the
// unique cell with x_i <= px < x_{i+1}, y_j <= py < y_{j+1}, so two binary
// searches over the accumulated corner arrays give the same cell.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_locate(StaticData sd_, SrcOpts so_, const double* __restrict__ spx,
                                                const double* __restrict__ spy, const double* __restrict__ cx_g,
                                                const double* __restrict__ cy_g, const double* __restrict__ ccx_g,
                                                const double* __restrict__ ccy_g, int* __restrict__ cell3,
                                                double* __restrict__ w3, int* __restrict__ mapped,
                                                int* __restrict__ pixmaps)
{
    extern __shared__ double sm[];
    const StaticData sd = eval_shape(sd_);
    const SrcOpts so = eval_grid(so_, sd_);
    const int snx = so.snx, sny = so.sny;
    double* cx = sm;
    double* cy = cx + snx + 1;
    double* ccx = cy + sny + 1;
    double* ccy = ccx + snx;
    for (int i = threadIdx.x; i <= snx; i += blockDim.x) cx[i] = cx_g[i];
    for (int j = threadIdx.x; j <= sny; j += blockDim.x) cy[j] = cy_g[j];
    for (int i = threadIdx.x; i < snx; i += blockDim.x) ccx[i] = ccx_g[i];
    for (int j = threadIdx.x; j < sny; j += blockDim.x) ccy[j] = ccy_g[j];
    __syncthreads();
    const double weight = 1.0 / sd.nsub;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < sd.n_sub; t += gridDim.x * blockDim.x) {
        double px = spx[t], py = spy[t];
        if (!(px >= cx[0] && px < cx[snx] && py >= cy[0] && py < cy[sny])) {
            cell3[3 * t] = -1; cell3[3 * t + 1] = -1; cell3[3 * t + 2] = -1;
            continue;
        }
        int lo = 0, hi = snx - 1;
        while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (cx[mid] <= px) lo = mid; else hi = mid - 1; }
        const int ci = lo;
        lo = 0; hi = sny - 1;
        while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (cy[mid] <= py) lo = mid; else hi = mid - 1; }
        const int cj = lo;
        const int xn = ((px > ccx[ci] && ci < snx - 1) || ci == 0) ? ci + 1 : ci - 1;
        const int yn = ((py > ccy[cj] && cj < sny - 1) || cj == 0) ? cj + 1 : cj - 1;
        const int c0 = cj * snx + ci, c1 = cj * snx + xn, c2 = yn * snx + ci;
        cell3[3 * t] = c0; cell3[3 * t + 1] = c1; cell3[3 * t + 2] = c2;
        mapped[c0] = 1; mapped[c1] = 1; mapped[c2] = 1;
        pixmaps[t / sd.nsub] = 1;
        const double p0x = ccx[ci], p0y = ccy[cj];
        const double p1x = ccx[xn], p1y = ccy[cj];
        const double p2x = ccx[ci], p2y = ccy[yn];
        const double d = (p0x - p1x) * (p1y - p2y) - (p1x - p2x) * (p0y - p1y);
        w3[3 * t]     = weight * (px * (p1y - p2y) + py * (p2x - p1x) + p1x * p2y - p1y * p2x) / d;
        w3[3 * t + 1] = weight * (px * (p2y - p0y) + py * (p0x - p2x) + p0y * p2x - p0x * p2y) / d;
        w3[3 * t + 2] = weight * (px * (p0y - p1y) + py * (p1x - p0x) + p0x * p1y - p0y * p1x) / d;
    }
}

void launch_locate(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st)
{
    cudaMemsetAsync(w.mapped, 0, sizeof(int) * so.snx * so.sny, st);
    cudaMemsetAsync(w.pixmaps, 0, sizeof(int) * (sd.n_mask > 0 ? sd.n_mask : 1), st);
    if (sd.n_sub == 0) return;
    size_t smem = sizeof(double) * (2 * (so.snx + so.sny) + 2);
    int blocks = (sd.n_sub + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_locate<<<blocks, 256, smem, st>>>(sd, so, w.spx, w.spy, w.cx, w.cy, w.ccx, w.ccy, w.cell3, w.w3, w.mapped,
                                        w.pixmaps);
    count_launches(1);
}

// ---------------------------------------------------------------------------
// Compaction (one block):
//   active source index: mapped cells in j-outer / i-inner order
//     (SourcePixel::assign_active_indices, pixelgrid.cpp:3590-3626)
//   active image pixels: masked pixels with >= 1 mapped sub-pixel, in the
//     masked-pixel order (assign_pixel_mappings, pixelgrid.cpp:12881-12910)
//   L row pointers: 3 entries per mapped sub-pixel (assign_Lmatrix 13298-13302)
// Block-wide exclusive scans over per-thread contiguous chunks keep the order.
// ---------------------------------------------------------------------------
__device__ int block_exclusive_scan(int v, int* warp_tot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int t = (lane < nw) ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_tot[lane] = t;   // inclusive warp totals
    }
    __syncthreads();
    int base = (warp > 0) ? warp_tot[warp - 1] : 0;
    int total = warp_tot[nw - 1];
    __syncthreads();
    warp_tot[32] = total;
    return base + x - v;
}

// The compaction runs on COMPACT_BLOCKS-way contiguous shares of the cells and
// of the masked pixels: k_compact_count counts, per share, the mapped cells,
// the active pixels and their L entries; k_compact_scan turns the counts into
// exclusive offsets (one block) and sets M, N, nnz; k_compact_write scans
// within each share and writes.  Shares and offsets keep the order.
__device__ __forceinline__ void compact_share(int len, int nshare, int b, int& b0, int& b1)
{
    const int per = (len + nshare - 1) / nshare;
    b0 = min(len, b * per);
    b1 = min(len, b0 + per);
}

__device__ __forceinline__ int pixel_entries(const int* __restrict__ cell3, int m, int nsub)
{
    int e = 0;
    for (int k = 0; k < nsub; k++) e += (cell3[3 * (m * nsub + k)] >= 0) ? 3 : 0;
    return e;
}

__global__ void __launch_bounds__(256) k_compact_count(StaticData sd_, SrcOpts so_, const int* __restrict__ mapped,
                                                       const int* __restrict__ cell3,
                                                       const int* __restrict__ pixmaps, int* __restrict__ cpart)
{
    const StaticData sd = eval_shape(sd_);
    const SrcOpts so = eval_grid(so_, sd_);
    __shared__ int red[3][8];
    const int nshare = gridDim.x, b = blockIdx.x;
    int c0, c1, p0, p1;
    compact_share(so.snx * so.sny, nshare, b, c0, c1);
    compact_share(sd.n_mask, nshare, b, p0, p1);
    int nc = 0, np = 0, ne = 0;
    for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) nc += mapped[k] ? 1 : 0;
    for (int m = p0 + threadIdx.x; m < p1; m += blockDim.x)
        if (pixmaps[m]) { np++; ne += pixel_entries(cell3, m, sd.nsub); }
    for (int o = 16; o > 0; o >>= 1) {
        nc += __shfl_xor_sync(0xffffffffu, nc, o);
        np += __shfl_xor_sync(0xffffffffu, np, o);
        ne += __shfl_xor_sync(0xffffffffu, ne, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][warp] = nc; red[1][warp] = np; red[2][warp] = ne; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int a0 = 0, a1 = 0, a2 = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a0 += red[0][k]; a1 += red[1][k]; a2 += red[2][k]; }
        cpart[b] = a0;
        cpart[1025 + b] = a1;
        cpart[2050 + b] = a2;
    }
}

__global__ void __launch_bounds__(1024) k_compact_scan(int nshare, int* __restrict__ cpart, int* __restrict__ rowptr,
                                                       GridState* gs)
{
    __shared__ int wt[33];
    __shared__ int tot[3];
    for (int a = 0; a < 3; a++) {
        int* v = cpart + 1025 * a;
        const int x = (threadIdx.x < nshare) ? v[threadIdx.x] : 0;
        const int off = block_exclusive_scan(x, wt);
        if (threadIdx.x == 0) tot[a] = wt[32];
        __syncthreads();
        if (threadIdx.x < nshare) v[threadIdx.x] = off;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int M = tot[0], N = tot[1];
        rowptr[N] = tot[2];
        gs->M = M;
        gs->N = N;
        gs->nnz = tot[2];
        if (M == 0) gs->status = QLP_ERR_NO_SOURCE_PIXELS;
    }
}

__global__ void __launch_bounds__(256) k_compact_write(StaticData sd_, SrcOpts so_, const int* __restrict__ mapped,
                                                       int* __restrict__ active_index, const int* __restrict__ cell3,
                                                       const int* __restrict__ pixmaps, int* __restrict__ rowidx,
                                                       int* __restrict__ pixindex, int* __restrict__ rowptr,
                                                       const int* __restrict__ cpart)
{
    const StaticData sd = eval_shape(sd_);
    const SrcOpts so = eval_grid(so_, sd_);
    __shared__ int wt[33];
    const int nshare = gridDim.x, b = blockIdx.x, T = blockDim.x;
    // ---- source cells: active index in cell order ----
    {
        int c0, c1;
        compact_share(so.snx * so.sny, nshare, b, c0, c1);
        const int chunk = (c1 - c0 + T - 1) / T;
        const int k0 = min(c1, c0 + (int)threadIdx.x * chunk), k1 = min(c1, k0 + chunk);
        int c = 0;
        for (int k = k0; k < k1; k++) c += mapped[k] ? 1 : 0;
        int off = cpart[b] + block_exclusive_scan(c, wt);
        for (int k = k0; k < k1; k++) active_index[k] = mapped[k] ? off++ : -1;
    }
    __syncthreads();
    // ---- image pixels: active rows in masked-pixel order, L row pointers ----
    {
        int p0, p1;
        compact_share(sd.n_mask, nshare, b, p0, p1);
        const int chunk = (p1 - p0 + T - 1) / T;
        const int m0 = min(p1, p0 + (int)threadIdx.x * chunk), m1 = min(p1, m0 + chunk);
        int c = 0, e = 0;
        for (int m = m0; m < m1; m++)
            if (pixmaps[m]) { c++; e += pixel_entries(cell3, m, sd.nsub); }
        int roff = cpart[1025 + b] + block_exclusive_scan(c, wt);
        __syncthreads();
        int eoff = cpart[2050 + b] + block_exclusive_scan(e, wt);
        for (int m = m0; m < m1; m++) {
            const int pix = sd.mpix[m];
            if (pixmaps[m]) {
                rowidx[m] = roff;
                pixindex[pix] = roff;
                rowptr[roff] = eoff;
                roff++;
                eoff += pixel_entries(cell3, m, sd.nsub);
            } else {
                rowidx[m] = -1;
                pixindex[pix] = -1;
            }
        }
    }
}

void launch_compact(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st)
{
    // pixels outside the mask keep -1 in pixindex
    cudaMemsetAsync(w.pixindex, 0xff, sizeof(int) * sd.nx * sd.ny, st);
    const int nshare = std::max(1, std::min(1024, std::max((sd.n_mask + 255) / 256, (so.snx * so.sny + 255) / 256)));
    k_compact_count<<<nshare, 256, 0, st>>>(sd, so, w.mapped, w.cell3, w.pixmaps, w.cpart);
    k_compact_scan<<<1, 1024, 0, st>>>(nshare, w.cpart, w.rowptr, w.gs);
    k_compact_write<<<nshare, 256, 0, st>>>(sd, so, w.mapped, w.active_index, w.cell3, w.pixmaps, w.rowidx,
                                            w.pixindex, w.rowptr, w.cpart);
    count_launches(3);
}

// ---------------------------------------------------------------------------
// L in CSR (assign_Lmatrix, pixelgrid.cpp:13259-13321): per active row, the
// mapped sub-pixels in sub-cell order, 3 entries each.  The same thread also
// writes the row with duplicate source indices merged (summed in CSR order,
// i.e. exactly the row of convert_Lmatrix_to_dense, pixelgrid.cpp:13734-13739),
// which the PSF kernel gathers from.
// ---------------------------------------------------------------------------
#define BUILD_L_MAXD 192      // entries of one row merged in local arrays (3 per sub-pixel, up to 8x8 split)

__global__ void __launch_bounds__(128) k_build_L(StaticData sd_, const int* __restrict__ rowidx,
                                                 const int* __restrict__ rowptr, const int* __restrict__ cell3,
                                                 const double* __restrict__ w3, const int* __restrict__ active_index,
                                                 int* __restrict__ Lidx, double* __restrict__ Lval,
                                                 int* __restrict__ cidx, double* __restrict__ cval,
                                                 int* __restrict__ ccnt)
{
    const StaticData sd = eval_shape(sd_);
    const int nsub = sd.nsub;
    if (3 * nsub <= BUILD_L_MAXD) {
        // one pass: each entry is written to the CSR row and merged at once
        // into the row's distinct cells, kept in this thread's local arrays
        // (a search over the distinct cells so far, not over all entries);
        // a cell's sum starts from 0.0 and adds its entries in CSR order, and
        // the distinct cells keep their first-occurrence order
        int di[BUILD_L_MAXD];
        double dv[BUILD_L_MAXD];
        for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < sd.n_mask; m += gridDim.x * blockDim.x) {
            const int r = rowidx[m];
            if (r < 0) continue;
            const int e0 = rowptr[r];
            int e = e0, nc = 0;
            for (int k = 0; k < nsub; k++) {
                const int t = m * nsub + k;
                const int c0 = cell3[3 * t];
                if (c0 < 0) continue;
                #pragma unroll
                for (int u = 0; u < 3; u++) {
                    const int idx = active_index[u == 0 ? c0 : cell3[3 * t + u]];
                    const double val = w3[3 * t + u];
                    Lidx[e] = idx;
                    Lval[e] = val;
                    e++;
                    int j = 0;
                    while (j < nc && di[j] != idx) j++;
                    if (j == nc) { di[nc] = idx; dv[nc] = 0.0 + val; nc++; }
                    else dv[j] += val;
                }
            }
            for (int j = 0; j < nc; j++) {
                cidx[e0 + j] = di[j];
                cval[e0 + j] = dv[j];
            }
            ccnt[r] = nc;
        }
        return;
    }
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < sd.n_mask; m += gridDim.x * blockDim.x) {
        const int r = rowidx[m];
        if (r < 0) continue;
        const int e0 = rowptr[r];
        int e = e0;
        for (int k = 0; k < nsub; k++) {
            const int t = m * nsub + k;
            if (cell3[3 * t] < 0) continue;
            for (int u = 0; u < 3; u++) {
                Lidx[e] = active_index[cell3[3 * t + u]];
                Lval[e] = w3[3 * t + u];
                e++;
            }
        }
        // merged row: first occurrence order, values summed in CSR order from 0
        int nc = 0;
        for (int a = e0; a < e; a++) {
            const int idx = Lidx[a];
            bool first = true;
            for (int b = e0; b < a; b++) if (Lidx[b] == idx) { first = false; break; }
            if (!first) continue;
            double v = 0.0;
            for (int b = a; b < e; b++) if (Lidx[b] == idx) v += Lval[b];
            cidx[e0 + nc] = idx;
            cval[e0 + nc] = v;
            nc++;
        }
        ccnt[r] = nc;
    }
}

void launch_build_L(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st)
{
    (void)so;
    if (sd.n_mask == 0) return;
    // a thread per masked pixel, each a long serial merge: 32-thread CTAs spread
    // the few warps over all SMs
    int blocks = (sd.n_mask + 31) / 32;
    k_build_L<<<blocks, 32, 0, st>>>(sd, w.rowidx, w.rowptr, w.cell3, w.w3, w.active_index, w.Lidx, w.Lval, w.cidx,
                                      w.cval, w.ccnt);
    count_launches(1);
}

}  // namespace qlpix
