// linalg.cu -- FP64 dense algebra of the inversion:
//   D = L'^T C^-1 d, F = L'^T C^-1 L' (SYRK), curvature R and F += lambda R,
//   blocked Cholesky of F and R, log det, the two triangular solves, the
//   model image, chi^2, s^T R s and the final -2 log(evidence).
// Reference: QLens::create_lensing_matrices_from_Lmatrix_dense
// (pixelgrid.cpp:15590-15736), add_regularization_term_to_dense_Fmatrix
// (15781-15819), invert_lens_mapping_dense (17346-17396), Cholesky_dcmp_packed
// (17071-17105), Cholesky_solve_lower_packed (17230-17246),
// Cholesky_logdet_lower_packed (17201-17210), Rmatrix_determinant_dense
// (18176-18191), calculate_image_pixel_surface_brightness_dense (18268-18290),
// calculate_regularization_prior_term (15821-15863), chi^2 and evidence
// assembly (lens.cpp:12950-13016, 12608-12615).
//
// Matrices are dense row-major with leading dimension ldF; the lower triangle
// holds F (and later its Cholesky factor).  Sizes past the active count M are
// padded to a multiple of 64 with an identity block, which leaves log det and
// the solution unchanged.  Every kernel reads N and M from the device-side
// GridState, so the launch sequence never waits for the host.
#include "qlpix_internal.h"
#include "chol.cuh"

namespace qlpix {

#define NB 64

__device__ __forceinline__ int mpad64(int M) { return (M + 63) & ~63; }

// ---- data and inverse-variance per active row ----
__global__ void k_dvec(StaticData sd, const GridState* __restrict__ gs, const int* __restrict__ rowpix,
                       double* __restrict__ dvec, double* __restrict__ cvec)
{
    const int N = gs->N;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        int pix = rowpix[r];
        dvec[r] = sd.data[pix];
        cvec[r] = sd.use_noise_map ? sd.covinv[pix] : sd.cov_inverse;
    }
}

void launch_dvec(const StaticData& sd, Work& w, int N_max, cudaStream_t st)
{
    if (N_max == 0) return;
    k_dvec<<<(N_max + 255) / 256, 256, 0, st>>>(sd, w.gs, w.rowpix, w.dvec, w.cvec);
    count_launches(1);
}

// ---- D = L'^T (C^-1 d): column sums over row chunks, then a fixed-order sum ----
#define D_CHUNK 256
__global__ void k_D_partial(const GridState* __restrict__ gs, const double* __restrict__ L, int ldL,
                            const double* __restrict__ dvec, const double* __restrict__ cvec,
                            double* __restrict__ part, int M_max)
{
    const int N = gs->N, M = gs->M;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const int r0 = blockIdx.y * D_CHUNK;
    if (col >= M || r0 >= N) return;
    const int r1 = min(r0 + D_CHUNK, N);
    double acc = 0;
    for (int r = r0; r < r1; r++) acc += L[(size_t)r * ldL + col] * dvec[r] * cvec[r];
    part[(size_t)blockIdx.y * M_max + col] = acc;
}

__global__ void k_D_final(const GridState* __restrict__ gs, const double* __restrict__ part, double* __restrict__ D,
                          int M_max)
{
    const int N = gs->N, M = gs->M;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= mpad64(M)) return;
    double acc = 0;
    if (col < M) {
        const int nch = (N + D_CHUNK - 1) / D_CHUNK;
        for (int c = 0; c < nch; c++) acc += part[(size_t)c * M_max + col];
    }
    D[col] = acc;
}

void launch_D(Work& w, int N_max, int M_max, cudaStream_t st)
{
    dim3 g((M_max + 127) / 128, (N_max + D_CHUNK - 1) / D_CHUNK);
    k_D_partial<<<g, 128, 0, st>>>(w.gs, w.Lpsf, w.ldL, w.dvec, w.cvec, w.partial, M_max);
    k_D_final<<<(w.ldF + 127) / 128, 128, 0, st>>>(w.gs, w.partial, w.D, M_max);
    count_launches(2);
}

// ---- F = L'^T C^-1 L', lower 64x64 tiles, FP64 ----
// nz[cb * nchunks + c] != 0 when rows [16 c, 16 c + 16) of L' have a nonzero in
// columns [64 cb, 64 cb + 64); one warp per (chunk, column block).
__global__ void __launch_bounds__(256) k_lpsf_nzflags(const GridState* __restrict__ gs,
                                                      const double* __restrict__ L, int ldL,
                                                      unsigned char* __restrict__ nz, int nchunks)
{
    const int N = gs->N, ncb = mpad64(gs->M) / NB;
    const int nch = (N + 15) / 16;
    const int lane = threadIdx.x & 31;
    const long task = (long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (task >= (long)nch * ncb) return;
    const int c = (int)(task % nch), cb = (int)(task / nch);
    bool any = false;
    for (int r = 16 * c; r < min(16 * c + 16, N); r++) {
        const double* row = L + (size_t)r * ldL + cb * NB;
        any |= (row[lane] != 0.0) | (row[lane + 32] != 0.0);
    }
    any = __any_sync(0xffffffffu, any);
    if (lane == 0) nz[(size_t)cb * nchunks + c] = any ? 1 : 0;
}

// A 16-pixel step whose rows of L' are zero in either tile's 64 columns adds
// only zero products, so it is skipped; the sums of the other steps run in
// the same order, so F is bit-for-bit the dense contraction's.
__global__ void __launch_bounds__(256) k_syrk64(const GridState* __restrict__ gs, const double* __restrict__ L,
                                                int ldL, const double* __restrict__ cvec, int use_noise_map,
                                                double cov_inverse, const unsigned char* __restrict__ nz, int nchunks,
                                                double* __restrict__ F, int ldF)
{
    __shared__ double As[16][NB + 1];
    __shared__ double Bs[16][NB + 1];
    int bi, bj;
    tri_index(blockIdx.x, bi, bj);
    const int N = gs->N, Mp = mpad64(gs->M);
    if (bi * NB >= Mp) return;
    const int a0 = bi * NB, b0 = bj * NB;
    const unsigned char* nza = nz + (size_t)bi * nchunks;
    const unsigned char* nzb = nz + (size_t)bj * nchunks;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0;
    for (int p0 = 0; p0 < N; p0 += 16) {
        if (!(nza[p0 >> 4] && nzb[p0 >> 4])) continue;       // uniform over the block
        #pragma unroll
        for (int e = 0; e < 4; e++) {
            int idx = threadIdx.x + e * 256;   // 0..1023 over 16 x 64
            int kk = idx >> 6, x = idx & 63;
            int p = p0 + kk;
            double va = 0, vb = 0;
            if (p < N) {
                va = L[(size_t)p * ldL + a0 + x];
                vb = L[(size_t)p * ldL + b0 + x];
                if (use_noise_map) vb *= cvec[p];
            }
            As[kk][x] = va;
            Bs[kk][x] = vb;
        }
        __syncthreads();
        #pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            double ra[4], rb[4];
            #pragma unroll
            for (int u = 0; u < 4; u++) ra[u] = As[kk][ty * 4 + u];
            #pragma unroll
            for (int v = 0; v < 4; v++) rb[v] = Bs[kk][tx * 4 + v];
            #pragma unroll
            for (int u = 0; u < 4; u++)
                #pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] += ra[u] * rb[v];
        }
        __syncthreads();
    }
    const double scale = use_noise_map ? 1.0 : cov_inverse;
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) F[(size_t)(a0 + ty * 4 + u) * ldF + b0 + tx * 4 + v] = acc[u][v] * scale;
}

void launch_syrk_fp64(const StaticData& sd, Work& w, int N_max, int M_max, cudaStream_t st)
{
    int nb = (M_max + NB - 1) / NB;
    int tiles = nb * (nb + 1) / 2;
    const long tasks = (long)((N_max + 15) / 16) * nb;
    k_lpsf_nzflags<<<(unsigned)((tasks + 7) / 8), 256, 0, st>>>(w.gs, w.Lpsf, w.ldL, w.lnz, w.lnz_chunks);
    k_syrk64<<<tiles, 256, 0, st>>>(w.gs, w.Lpsf, w.ldL, w.cvec, sd.use_noise_map, sd.cov_inverse, w.lnz,
                                    w.lnz_chunks, w.F, w.ldF);
    count_launches(2);
}

// ---- curvature R (dense lower) and F += lambda R ----
// R = Hx^T Hx + Hy^T Hy with Hx rows (-2 at a, +1 at active x-neighbours) and
// Hy likewise (SourcePixel::generate_hmatrices, pixelgrid.cpp:2968-3071;
// generate_Rmatrix_from_hmatrices 3073-3240).  In closed form per active cell:
// diagonal 8 + #active 4-neighbours, -4 for an active +-1 neighbour, +1 for an
// active +-2 neighbour whose middle cell is active.
__device__ __forceinline__ int act_at(const int* ai, int snx, int sny, int i, int j)
{
    if (i < 0 || j < 0 || i >= snx || j >= sny) return -1;
    return ai[j * snx + i];
}

__global__ void k_reg(const GridState* __restrict__ gs, const int* __restrict__ ai,
                      const double* __restrict__ regp, double* __restrict__ F, double* __restrict__ R, int ldF,
                      int do_reg, int parts)
{
    const bool toF = parts & REG_F, toR = parts & REG_R;
    const double regparam = *regp;
    const int snx = gs->snx, sny = gs->sny;
    const int M = gs->M, Mp = mpad64(M);
    const int ncell = snx * sny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell + (Mp - M); c += gridDim.x * blockDim.x) {
        if (c >= ncell) {   // identity padding
            int i = M + (c - ncell);
            if (toF) F[(size_t)i * ldF + i] = 1.0;
            if (do_reg && toR) R[(size_t)i * ldF + i] = 1.0;
            continue;
        }
        if (!do_reg) continue;
        const int a = ai[c];
        if (a < 0) continue;
        const int ci = c % snx, cj = c / snx;
        int nb1[4] = {act_at(ai, snx, sny, ci + 1, cj), act_at(ai, snx, sny, ci - 1, cj),
                      act_at(ai, snx, sny, ci, cj + 1), act_at(ai, snx, sny, ci, cj - 1)};
        int nb2[4] = {act_at(ai, snx, sny, ci + 2, cj), act_at(ai, snx, sny, ci - 2, cj),
                      act_at(ai, snx, sny, ci, cj + 2), act_at(ai, snx, sny, ci, cj - 2)};
        double diag = 8.0;
        for (int k = 0; k < 4; k++) if (nb1[k] >= 0) diag += 1.0;
        if (toR) R[(size_t)a * ldF + a] = diag;
        if (toF) F[(size_t)a * ldF + a] += regparam * diag;
        for (int k = 0; k < 4; k++) {
            int b = nb1[k];
            if (b >= 0 && b < a) {
                if (toR) R[(size_t)a * ldF + b] = -4.0;
                if (toF) F[(size_t)a * ldF + b] += regparam * -4.0;
            }
            int b2 = nb2[k];
            if (b2 >= 0 && nb1[k] >= 0 && b2 < a) {
                if (toR) R[(size_t)a * ldF + b2] = 1.0;
                if (toF) F[(size_t)a * ldF + b2] += regparam * 1.0;
            }
        }
    }
}

void launch_regularization(const SrcOpts& so, Work& w, int M_max, const double* regp, int parts, cudaStream_t st)
{
    const int ncell = so.snx * so.sny;
    if (so.regularization && (parts & REG_R)) cudaMemsetAsync(w.R, 0, sizeof(double) * (size_t)w.ldF * w.ldF, st);
    int total = ncell + 64;
    k_reg<<<(total + 255) / 256, 256, 0, st>>>(w.gs, w.active_index, regp, w.F, w.R, w.ldF, so.regularization,
                                               parts);
    count_launches(1);
    (void)M_max;
}

// ---- Cholesky, log det and solve: the templates of chol.cuh in FP64 ----
// Attributes are per translation unit: each .cu has its own instance of a
// kernel template, so mixed.cu sets those of its float instances itself.
void linalg_init_attributes()
{
    solve_init_attributes<double>();
}


int launch_cholesky_fp64(double* A, int ld, int M_max, const GridState* gs, int which, double* linv, cudaStream_t st)
{
    return launch_cholesky_t<double>(A, ld, M_max, gs, which, st, linv);
}

void launch_logdet(const double* A, int ld, int M_max, Work& w, int which, cudaStream_t st)
{
    (void)M_max;
    k_logdet_t<double><<<1, 1024, 0, st>>>(A, ld, w.gs, w.out, which);
    count_launches(1);
}

void launch_solve_fp64(Work& w, int M_max, cudaStream_t st)
{
    (void)M_max;
    k_solve_t<double><<<1, 1024, solve_smem_bytes<double>(w.ldF), st>>>(w.F, w.ldF, w.linv, w.gs, w.D, w.s, w.ldF);
    count_launches(1);
}

// ---- model image, chi^2, s^T R s and the evidence ----
__global__ void __launch_bounds__(256) k_model(const GridState* __restrict__ gs, const double* __restrict__ L,
                                               int ldL, const double* __restrict__ s, double* __restrict__ model)
{
    const int N = gs->N, M = gs->M;
    const int lane = threadIdx.x & 31;
    for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < N; r += gridDim.x * (blockDim.x >> 5)) {
        const double* row = L + (size_t)r * ldL;
        double acc = 0;
        for (int c = lane; c < M; c += 32) acc += row[c] * s[c];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) model[r] = acc;
    }
}

__global__ void __launch_bounds__(1024) k_final(StaticData sd_, SrcOpts so_, const GridState* __restrict__ gs,
                                                const int* __restrict__ rowidx, const double* __restrict__ model,
                                                const double* __restrict__ s, const int* __restrict__ ai,
                                                const double* __restrict__ regp, EvalOut* out)
{
    const StaticData sd = eval_shape(sd_);
    const SrcOpts so = eval_grid(so_, sd_);
    const double regparam = *regp;
    __shared__ double red[4][32];
    const int M = gs->M;
    double chi = 0, es = 0, chi_act = 0, logc = 0;
    for (int m = threadIdx.x; m < sd.n_mask; m += blockDim.x) {
        const int pix = sd.mpix[m];
        const double c = sd.use_noise_map ? sd.covinv[pix] : sd.cov_inverse;
        const int r = rowidx[m];
        double dd = (r >= 0) ? model[r] - sd.data[pix] : sd.data[pix];
        chi += dd * dd * c;
        if (r >= 0) chi_act += dd * dd * c;     // the pixels the lambda optimisation's chi^2 runs over
        if (r >= 0 && sd.noise_term && sd.use_noise_map) logc += log(c);
    }
    if (so.regularization && regparam != 0) {
        const int snx = so.snx, sny = so.sny;
        for (int cidx = threadIdx.x; cidx < snx * sny; cidx += blockDim.x) {
            const int a = ai[cidx];
            if (a < 0) continue;
            const int ci = cidx % snx, cj = cidx / snx;
            int nb1[4] = {act_at(ai, snx, sny, ci + 1, cj), act_at(ai, snx, sny, ci - 1, cj),
                          act_at(ai, snx, sny, ci, cj + 1), act_at(ai, snx, sny, ci, cj - 1)};
            int nb2[4] = {act_at(ai, snx, sny, ci + 2, cj), act_at(ai, snx, sny, ci - 2, cj),
                          act_at(ai, snx, sny, ci, cj + 2), act_at(ai, snx, sny, ci, cj - 2)};
            double diag = 8.0, rs = 0;
            for (int k = 0; k < 4; k++) {
                if (nb1[k] >= 0) { diag += 1.0; rs += -4.0 * s[nb1[k]]; }
                if (nb2[k] >= 0 && nb1[k] >= 0) rs += s[nb2[k]];
            }
            rs += diag * s[a];
            es += s[a] * rs;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        chi += __shfl_xor_sync(0xffffffffu, chi, o);
        es += __shfl_xor_sync(0xffffffffu, es, o);
        chi_act += __shfl_xor_sync(0xffffffffu, chi_act, o);
        logc += __shfl_xor_sync(0xffffffffu, logc, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = chi;
        red[1][threadIdx.x >> 5] = es;
        red[2][threadIdx.x >> 5] = chi_act;
        red[3][threadIdx.x >> 5] = logc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double c2 = 0, e2 = 0, ca = 0, lc = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            c2 += red[0][k]; e2 += red[1][k]; ca += red[2][k]; lc += red[3][k];
        }
        double regterms = 0, loglike = 0;
        if (so.regularization && M > 0) {
            if (regparam != 0) {
                regterms = regparam * e2 - M * log(regparam) - out->logdet_R;
                loglike += regterms;
            }
            loglike += out->logdet_F;
        }
        loglike += c2;
        // the pixel-noise normalisation, QLens 'include_noise_term_in_loglike'
        // (lens.cpp:13033-13043): minus the log of C^-1 over the active pixels
        // with a noise map, or the masked-pixel count times log(1/sigma^2)
        // without one, plus the masked-pixel count times log(2 pi)
        if (sd.noise_term) {
            loglike -= sd.use_noise_map ? lc : sd.n_mask * log(sd.cov_inverse);
            loglike += sd.n_mask * log(6.28318530717958647692);
        }
        int status = gs->status;
        if (status == 0 && (gs->not_spd_F || gs->not_spd_R)) status = QLP_ERR_NOT_SPD;
        // QLens::chisq_regparam_dense (pixelgrid.cpp:16688-16692): Ed + prior + log det F
        out->f_regopt = ca + ((so.regularization && M > 0) ? ((regparam != 0 ? regterms : 0.0) + out->logdet_F) : 0.0);
        out->chisq0 = c2;
        out->Es_times_two = e2;
        out->regterms = regterms;
        out->m2logev = (status == QLP_ERR_NO_SOURCE_PIXELS) ? 2e30 : loglike;
        out->n_active_pixels = gs->N;
        out->n_active_src = M;
        out->L_nnz = gs->nnz;
        out->status = status;
    }
}

void launch_model_chi2(const StaticData& sd, const SrcOpts& so, Work& w, int N_max, int M_max, const double* regp,
                       cudaStream_t st, bool model_ready)
{
    (void)M_max;
    if (N_max > 0 && !model_ready) {
        int blocks = (N_max + 7) / 8;
        if (blocks > 152 * 16) blocks = 152 * 16;
        k_model<<<blocks, 256, 0, st>>>(w.gs, w.Lpsf, w.ldL, w.s, w.model);
    }
    k_final<<<1, 1024, 0, st>>>(sd, so, w.gs, w.rowidx, w.model, w.s, w.active_index, regp, w.out);
    count_launches(2);
}

}  // namespace qlpix
