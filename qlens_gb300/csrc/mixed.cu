// mixed.cu -- mixed-precision inversion: TF32 tensor-core SYRK (3xTF32 split),
// FP32 Cholesky of F and R, FP64 log det accumulation and FP64 iterative
// refinement of the source amplitudes.
//
//   L'32   = P L accumulated in FP32 (psf.cu)                   only feeds F
//   X      = (L'32 * sqrt(C^-1))^T split into TF32 hi + lo      k_convert_x
//   F32    = X X^T on tcgen05 (block-sparse over pixel blocks)   k_syrk_tc
//   F32   += lambda R, R32 = R                                  k_reg32
//   L_F L_F^T = F32, L_R L_R^T = R32 (FP32 blocked Cholesky)    chol.cuh
//   log det F, log det R: 2 sum log diag, accumulated in FP64
//   D = L^T P^T (C^-1 d)                     (FP64, sparseops.cu)
//   s = F32^-1 D, then twice: r = D - L^T P^T C^-1 P L s - lambda R s (FP64),
//                              s += F32^-1 r
//   model = P L s                             (FP64, for chi^2)
// The plain FP64 path (linalg.cu) computes the same quantities entirely in
// FP64; the mixed path's deviation from it is measured by the tests.
#include <cuda.h>
#include <cstring>
#include "qlpix_ctx.h"
#include "chol.cuh"
#include "tc_syrk.cuh"

namespace qlpix {

struct MixedWork {
    float* L32 = nullptr;    // N_cap x ld32 PSF-convolved L, FP32
    double* t = nullptr;     // N (image-plane scratch)
    float* X_hi = nullptr;
    float* X_lo = nullptr;
    int K_cap = 0;           // columns of X (image pixels), multiple of 32
    int M_cap = 0;           // rows of X, multiple of 128
    unsigned char* nz = nullptr;
    int nkb_cap = 0;
    float* F32 = nullptr;
    float* R32 = nullptr;
    int ld32 = 0;
    double* u = nullptr;     // N
    double* v = nullptr;     // M
    double* r = nullptr;     // M
    double* z = nullptr;     // M
    double* y = nullptr;     // M (solve scratch)
    double* part = nullptr;
    float* linvF = nullptr;  // inverses of the 64x64 diagonal Cholesky blocks
    float* linvR = nullptr;
    CUtensorMap map_hi, map_lo;
    bool ready = false;
};

static MixedWork* mw_of(Slot& s) { return reinterpret_cast<MixedWork*>(s.mixed); }

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

static int make_map(CUtensorMap* map, float* base, int rows, int cols)
{
    EncodeTiledFn enc = get_encode();
    if (!enc) return QLP_ERR_CUDA;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(float)};
    cuuint32_t box[2] = {TC_KB, TC_TILE};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? QLP_OK : QLP_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// X = (L' sqrt(c))^T as TF32 hi + lo, and the nonzero flags of 128x32 blocks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float to_tf32(float f)
{
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(f));
    return __uint_as_float(u);
}

__global__ void __launch_bounds__(256) k_convert_x(const GridState* __restrict__ gs, const float* __restrict__ L,
                                                   int ldL, const double* __restrict__ cvec, float* __restrict__ Xh,
                                                   float* __restrict__ Xl, int K_cap, unsigned char* __restrict__ nz,
                                                   int nkb_cap)
{
    __shared__ float th[32][33];
    __shared__ float tl[32][33];
    const int N = gs->N, M = gs->M;
    const int Mp = (M + TC_TILE - 1) / TC_TILE * TC_TILE;
    const int Np = (N + TC_KB - 1) / TC_KB * TC_KB;
    const int p0 = blockIdx.x * 32, a0 = blockIdx.y * 32;
    if (p0 >= Np || a0 >= Mp) return;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    __shared__ float sq[32];
    if (threadIdx.x < 32) sq[threadIdx.x] = (p0 + threadIdx.x < N) ? (float)sqrt(cvec[p0 + threadIdx.x]) : 0.0f;
    __syncthreads();
    bool any = false;
    for (int k = ty; k < 32; k += 8) {
        const int p = p0 + k, a = a0 + tx;
        float x = 0;
        if (p < N && a < M) x = L[(size_t)p * ldL + a] * sq[k];
        const float h = to_tf32(x);
        const float l = to_tf32(x - h);   // exact: h is x rounded to fewer bits
        th[k][tx] = h;
        tl[k][tx] = l;
        any |= (x != 0.0f);
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int a = a0 + k, p = p0 + tx;
        Xh[(size_t)a * K_cap + p] = th[tx][k];
        Xl[(size_t)a * K_cap + p] = tl[tx][k];
    }
    const int anyb = __syncthreads_or(any ? 1 : 0);
    if (threadIdx.x == 0 && anyb) nz[(size_t)(a0 / TC_TILE) * nkb_cap + p0 / TC_KB] = 1;
}

// F32 += lambda R; R32 = R; identity beyond M up to the 64-padding.
__device__ __forceinline__ int act_at32(const int* ai, int snx, int sny, int i, int j)
{
    if (i < 0 || j < 0 || i >= snx || j >= sny) return -1;
    return ai[j * snx + i];
}

__global__ void k_reg32(const GridState* __restrict__ gs, const int* __restrict__ ai, int snx, int sny,
                        double regparam, float* __restrict__ F, float* __restrict__ R, int ld, int do_reg)
{
    const int M = gs->M, Mp = (M + 63) & ~63;
    const int ncell = snx * sny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell + (Mp - M); c += gridDim.x * blockDim.x) {
        if (c >= ncell) {
            int i = M + (c - ncell);
            F[(size_t)i * ld + i] = 1.0f;
            if (do_reg) R[(size_t)i * ld + i] = 1.0f;
            continue;
        }
        if (!do_reg) continue;
        const int a = ai[c];
        if (a < 0) continue;
        const int ci = c % snx, cj = c / snx;
        int nb1[4] = {act_at32(ai, snx, sny, ci + 1, cj), act_at32(ai, snx, sny, ci - 1, cj),
                      act_at32(ai, snx, sny, ci, cj + 1), act_at32(ai, snx, sny, ci, cj - 1)};
        int nb2[4] = {act_at32(ai, snx, sny, ci + 2, cj), act_at32(ai, snx, sny, ci - 2, cj),
                      act_at32(ai, snx, sny, ci, cj + 2), act_at32(ai, snx, sny, ci, cj - 2)};
        double diag = 8.0;
        for (int k = 0; k < 4; k++) if (nb1[k] >= 0) diag += 1.0;
        R[(size_t)a * ld + a] = (float)diag;
        F[(size_t)a * ld + a] = (float)((double)F[(size_t)a * ld + a] + regparam * diag);
        for (int k = 0; k < 4; k++) {
            int b = nb1[k];
            if (b >= 0 && b < a) {
                R[(size_t)a * ld + b] = -4.0f;
                F[(size_t)a * ld + b] = (float)((double)F[(size_t)a * ld + b] - 4.0 * regparam);
            }
            int b2 = nb2[k];
            if (b2 >= 0 && nb1[k] >= 0 && b2 < a) {
                R[(size_t)a * ld + b2] = 1.0f;
                F[(size_t)a * ld + b2] = (float)((double)F[(size_t)a * ld + b2] + regparam);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 refinement pieces
// ---------------------------------------------------------------------------
__global__ void k_copy_init(const GridState* __restrict__ gs, const double* __restrict__ D, double* __restrict__ r,
                            double* __restrict__ s)
{
    const int Mp = (gs->M + 63) & ~63;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Mp; i += gridDim.x * blockDim.x) {
        r[i] = D[i];
        s[i] = 0.0;
    }
}

__global__ void k_axpy(const GridState* __restrict__ gs, const double* __restrict__ z, double* __restrict__ s)
{
    const int Mp = (gs->M + 63) & ~63;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Mp; i += gridDim.x * blockDim.x) s[i] += z[i];
}

// r = D - v - lambda R s   (v = L'^T C^-1 L' s; R applied by its stencil)
__global__ void k_residual(const GridState* __restrict__ gs, const double* __restrict__ D,
                           const double* __restrict__ vv, const int* __restrict__ ai, int snx, int sny,
                           double regparam, int do_reg, const double* __restrict__ s, double* __restrict__ r)
{
    const int M = gs->M;
    const int ncell = snx * sny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        const int a = ai[c];
        if (a < 0) continue;
        const double v = vv[a];
        double rs = 0;
        if (do_reg) {
            const int ci = c % snx, cj = c / snx;
            int nb1[4] = {act_at32(ai, snx, sny, ci + 1, cj), act_at32(ai, snx, sny, ci - 1, cj),
                          act_at32(ai, snx, sny, ci, cj + 1), act_at32(ai, snx, sny, ci, cj - 1)};
            int nb2[4] = {act_at32(ai, snx, sny, ci + 2, cj), act_at32(ai, snx, sny, ci - 2, cj),
                          act_at32(ai, snx, sny, ci, cj + 2), act_at32(ai, snx, sny, ci, cj - 2)};
            double diag = 8.0;
            for (int k = 0; k < 4; k++) {
                if (nb1[k] >= 0) { diag += 1.0; rs += -4.0 * s[nb1[k]]; }
                if (nb2[k] >= 0 && nb1[k] >= 0) rs += s[nb2[k]];
            }
            rs += diag * s[a];
        }
        r[a] = D[a] - v - regparam * rs;
    }
    (void)M;
}

// ---------------------------------------------------------------------------
void mixed_free(Slot& c)
{
    MixedWork* m = mw_of(c);
    if (!m) return;
    void* ptrs[] = {m->L32, m->t, m->X_hi, m->X_lo, m->nz, m->F32, m->R32, m->u, m->v, m->r, m->z, m->y, m->part,
                    m->linvF, m->linvR};
    for (void* p : ptrs) if (p) cudaFree(p);
    delete m;
    c.mixed = nullptr;
}

int mixed_init(Slot& c)
{
    MixedWork* m = mw_of(c);
    const int M_cap = (c.M_cap + TC_TILE - 1) / TC_TILE * TC_TILE;
    const int K_cap = (c.N_cap + TC_KB - 1) / TC_KB * TC_KB + TC_KB;
    if (m && m->ready && m->M_cap >= M_cap && m->K_cap >= K_cap) return QLP_OK;
    mixed_free(c);
    m = new MixedWork();
    c.mixed = m;
    m->M_cap = M_cap;
    m->K_cap = K_cap;
    m->nkb_cap = K_cap / TC_KB;
    m->ld32 = M_cap;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes > 0 ? bytes : 16); };
    A((void**)&m->X_hi, sizeof(float) * (size_t)M_cap * K_cap);
    A((void**)&m->X_lo, sizeof(float) * (size_t)M_cap * K_cap);
    A((void**)&m->nz, (size_t)(M_cap / TC_TILE) * m->nkb_cap);
    A((void**)&m->F32, sizeof(float) * (size_t)M_cap * M_cap);
    A((void**)&m->R32, sizeof(float) * (size_t)M_cap * M_cap);
    A((void**)&m->L32, sizeof(float) * (size_t)c.N_cap * M_cap);
    A((void**)&m->t, sizeof(double) * (size_t)(c.N_cap + 64));
    A((void**)&m->u, sizeof(double) * (size_t)(c.N_cap + 64));
    A((void**)&m->v, sizeof(double) * M_cap);
    A((void**)&m->r, sizeof(double) * M_cap);
    A((void**)&m->z, sizeof(double) * M_cap);
    A((void**)&m->y, sizeof(double) * M_cap);
    A((void**)&m->part, sizeof(double) * (size_t)M_cap * (ltw_chunks(c.N_cap) + 1));
    A((void**)&m->linvF, sizeof(float) * (size_t)M_cap * 64);
    A((void**)&m->linvR, sizeof(float) * (size_t)M_cap * 64);
    if (e != cudaSuccess) {
        set_error("%s (%d)", "mixed-precision workspace allocation failed", (int)e);
        return QLP_ERR_NOMEM;
    }
    cudaMemset(m->X_hi, 0, sizeof(float) * (size_t)M_cap * K_cap);
    cudaMemset(m->X_lo, 0, sizeof(float) * (size_t)M_cap * K_cap);
    if (make_map(&m->map_hi, m->X_hi, M_cap, K_cap) != QLP_OK || make_map(&m->map_lo, m->X_lo, M_cap, K_cap) != QLP_OK) {
        set_error("%s (%d)", "cuTensorMapEncodeTiled unavailable or failed", 0);
        return QLP_ERR_CUDA;
    }
    cudaFuncSetAttribute(k_syrk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    cudaFuncSetAttribute(k_chol_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, UPD_SMEM);
    solve_init_attributes<float>();
    m->ready = true;
    return QLP_OK;
}

// FP32 blocked Cholesky for the mixed path: shared-memory potrf of each 64x64
// diagonal tile, per-row triangular solve of the tiles below it, the trailing
// update on the tensor cores, then all diagonal inverses in one launch.
static int cholesky_mixed(float* A, int ld, int M_cap, GridState* gs, int which, cudaStream_t st, float* Linv)
{
    const int nbm = (M_cap + CB - 1) / CB;
    int n = 0;
    for (int k = 0; k < nbm; k++) {
        const int rem = nbm - k - 1;
        k_potrf_t<float><<<1, 256, 0, st>>>(A, ld, k, gs, which, nullptr);
        n++;
        if (rem > 0) {
            k_trsm_rows<<<rem, CB, 0, st>>>(A, ld, k, gs);
            const int nt = (rem * CB + TC_TILE - 1) / TC_TILE;
            k_chol_update_tc<<<nt * (nt + 1) / 2, 128, UPD_SMEM, st>>>(A, ld, k, gs);
            n += 2;
        }
    }
    k_diag_inverse<float><<<nbm, CB, 0, st>>>(A, ld, gs, Linv);
    n++;
    count_launches(n);
    return n;
}

int run_inversion_mixed(Slot& slot, const StaticData& sd, const SrcOpts& so, double regparam, cudaStream_t st,
                        cudaEvent_t* ev)
{
    int rc = mixed_init(slot);
    if (rc != QLP_OK) return rc;
    MixedWork* m = mw_of(slot);
    Work& w = slot.w;
    const int N_cap = sd.n_mask;
    const int Mc = slot.M_cap;
    int n = 0;

    // D = L^T P^T (C^-1 d), FP64
    op_conv(sd, w, N_cap, true, w.dvec, w.cvec, m->t, st);
    op_LTw(w, N_cap, m->M_cap, m->t, m->part, w.D, st);
    // L'32, then X and the block flags
    launch_psf32(sd, w, m->L32, m->ld32, m->M_cap, st);
    cudaMemsetAsync(m->nz, 0, (size_t)(m->M_cap / TC_TILE) * m->nkb_cap, st);
    {
        dim3 g(m->K_cap / 32, m->M_cap / 32);
        k_convert_x<<<g, 256, 0, st>>>(w.gs, m->L32, m->ld32, w.cvec, m->X_hi, m->X_lo, m->K_cap, m->nz, m->nkb_cap);
        n++;
    }
    if (ev) cudaEventRecord(ev[3], st);
    {
        const int nt = m->M_cap / TC_TILE;
        k_syrk_tc<<<nt * (nt + 1) / 2, 128, TC_SMEM, st>>>(m->map_hi, m->map_lo, w.gs, m->nz, m->nkb_cap, m->F32,
                                                            m->ld32);
        n++;
    }
    if (ev) cudaEventRecord(ev[4], st);
    if (so.regularization) cudaMemsetAsync(m->R32, 0, sizeof(float) * (size_t)m->ld32 * m->ld32, st);
    k_reg32<<<(so.snx * so.sny + 64 + 255) / 256, 256, 0, st>>>(w.gs, w.active_index, so.snx, so.sny, regparam,
                                                                m->F32, m->R32, m->ld32, so.regularization);
    n++;
    if (so.regularization) {
        n += cholesky_mixed(m->R32, m->ld32, Mc, w.gs, 1, st, m->linvR);
        k_logdet_t<float><<<1, 1024, 0, st>>>(m->R32, m->ld32, w.gs, w.out, 1);
        n++;
    }
    n += cholesky_mixed(m->F32, m->ld32, Mc, w.gs, 0, st, m->linvF);
    k_logdet_t<float><<<1, 1024, 0, st>>>(m->F32, m->ld32, w.gs, w.out, 0);
    n++;
    // s = F^-1 D with two FP64 refinement sweeps
    k_copy_init<<<(Mc + 255) / 256, 256, 0, st>>>(w.gs, w.D, m->r, w.s);
    n++;
    const int refine = 2;
    for (int it = 0; it <= refine; it++) {
        k_solve_t<float><<<1, 1024, solve_smem_bytes<float>(Mc), st>>>(m->F32, m->ld32, m->linvF, w.gs, m->r, m->z,
                                                                      Mc);
        k_axpy<<<(Mc + 255) / 256, 256, 0, st>>>(w.gs, m->z, w.s);
        n += 2;
        if (it == refine) break;
        op_Ls(w, N_cap, w.s, m->t, st);
        op_conv(sd, w, N_cap, false, m->t, nullptr, m->u, st);
        op_conv(sd, w, N_cap, true, m->u, w.cvec, m->t, st);
        op_LTw(w, N_cap, m->M_cap, m->t, m->part, m->v, st);
        k_residual<<<(so.snx * so.sny + 255) / 256, 256, 0, st>>>(w.gs, w.D, m->v, w.active_index, so.snx, so.sny,
                                                                  regparam, so.regularization, w.s, m->r);
        n++;
    }
    // model image P L s in FP64 for chi^2
    op_Ls(w, N_cap, w.s, m->t, st);
    op_conv(sd, w, N_cap, false, m->t, nullptr, w.model, st);
    count_launches(n);
    return QLP_OK;
}

}  // namespace qlpix
