// mixed.cu -- mixed-precision inversion: TF32 tensor-core SYRK (3xTF32 split),
// FP32 Cholesky of F and R, FP64 log det accumulation and FP64 iterative
// refinement of the source amplitudes.
//
//   X      = (P L sqrt(C^-1))^T, built column by column (one source cell
//            per CTA, exact fixed-point sums), split into TF32 hi + lo  k_psf_x
//   F32    = X X^T on tcgen05 (block-sparse over pixel blocks)   k_syrk_tc
//   F32   += lambda R, R32 = R                                  k_reg32
//   L_F L_F^T = F32, L_R L_R^T = R32 (FP32 blocked Cholesky)    chol.cuh
//   log det F, log det R: 2 sum log diag, accumulated in FP64
//   D = L^T P^T (C^-1 d)                     (FP64; L^T from L by source cell)
//   s = F32^-1 D, then `refine` times: r = D - L^T P^T C^-1 P L s - lambda R s (FP64),
//                                       s += F32^-1 r
//   model = P L s                             (FP64, for chi^2)
// The plain FP64 path (linalg.cu) computes the same quantities entirely in
// FP64; the mixed path's deviation from it is measured by the tests.
#include <cuda.h>
#include <cuda_fp16.h>
#include <climits>
#include <cstring>
#include <algorithm>
#include "qlpix_ctx.h"
#include "chol.cuh"
#include "tc_syrk.cuh"
#include "chol128.cuh"

namespace qlpix {

struct MixedWork {
    double* t = nullptr;     // N (image-plane scratch)
    // L by source cell (CSC of the merged pre-PSF rows), for k_psf_x
    int* colcnt = nullptr;   // M_cap + 1 counts, then the column pointers
    int* cursor = nullptr;   // M_cap
    int* colrow = nullptr;   // nnz_cap
    float* colval = nullptr; // nnz_cap
    float* sqc = nullptr;    // N_cap: sqrt(C^-1) per active row
    int nnz_cap = 0;
    int2* pixT = nullptr;    // image pixels, x fastest: (active row or -1, sqrt(C^-1))
    float* F0 = nullptr;     // lambda optimisation: X X^T before lambda R (allocated on first use)
    int* col_u = nullptr;    // nnz_cap: rows of each column in atomic (fill) order
    int* src_u = nullptr;    // nnz_cap: their positions in the merged CSR rows
    double* colval64 = nullptr; // nnz_cap: FP64 values, rows ascending within a column
    void* X_hi = nullptr;    // F16 (or TF32 in FP32 storage) parts of X
    void* X_lo = nullptr;
    bool half = true;        // X in F16 for the kind::f16 SYRK
    int K_cap = 0;           // columns of X (image pixels), multiple of 32
    int M_cap = 0;           // rows of X, multiple of 128
    unsigned char* nz = nullptr;
    int nkb_cap = 0;
    int4* psfx_meta = nullptr; // band schedule: 2 int4 per (cell, band) item (k_psfx_meta)
    int psfx_bands = 0;        // bands it has room for
    float* F32 = nullptr;
    float* R32 = nullptr;
    int ld32 = 0;
    double* u = nullptr;     // N
    double* v = nullptr;     // M
    double* r = nullptr;     // M
    double* z = nullptr;     // M
    double* y = nullptr;     // M (solve scratch)
    double* img = nullptr;   // npix_pad: dense padded image for the FP64 convolutions
    float* linvF = nullptr;  // per 128-block of F: inverse of its diagonal factor, then its transpose
    float* linv128 = nullptr; // the same for R's current diagonal block
    float* yf = nullptr;     // M_cap: forward-solve result
    float* zf = nullptr;     // M_cap: backward-solve result (FP32 copy read by other CTAs)
    int* flags = nullptr;    // 2 x nb: per-block "published" flags of the two sweeps
    int nb = 0;              // 128-blocks of M_cap
    CUtensorMap map_hi, map_lo;
    // the Cholesky's current panel, split for its trailing update (k_chol_upd16):
    // F16 hi + lo [M_cap][128] and the scale exponent of each row;
    // one set for F, one for R (factored concurrently on the side stream)
    __half* Pf_hi = nullptr; __half* Pf_lo = nullptr; int* Pf_exp = nullptr;
    __half* Pr_hi = nullptr; __half* Pr_lo = nullptr; int* Pr_exp = nullptr;
    CUtensorMap map_pf_hi, map_pf_lo, map_pr_hi, map_pr_lo;
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

// 128-row boxes of 128 bytes (32 FP32 or 64 F16 values), 128-byte swizzle
static int make_map(CUtensorMap* map, void* base, int rows, int cols, bool half)
{
    EncodeTiledFn enc = get_encode();
    if (!enc) return QLP_ERR_CUDA;
    const size_t esz = half ? 2 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * esz};
    cuuint32_t box[2] = {(cuuint32_t)(128 / esz), TC_TILE};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, half ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims,
                     strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? QLP_OK : QLP_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// X = (P L sqrt(C^-1))^T as TF32 hi + lo, and the nonzero flags of its
// 128-cell x 32-pixel blocks, built one source cell (one row of X) at a time.
//
// Row s of X is the PSF-convolved image of source cell s: every pixel q that
// sees s (column s of the pre-PSF L) spreads L[q][s] over its PSF neighbours
// p with weight psf[k][l] (the transpose of QLens's gather,
// pixelgrid.cpp:14126-14168); the sum at p is then scaled by sqrt(C^-1) of p.
// The sums are accumulated as 64-bit fixed point in shared memory, so they
// are exact and independent of the order the atomics land in (the result is
// the same bits every run): each product is the exact product of two 32-bit
// integers, the tap on its grid (StaticData::psf_int) and the L entry on the
// grid 2^-PSFX_LEXP (2^-28: 4e-9 absolute, far below FP32 resolution of the
// entries) -- one wide multiply per tap.  No dense L' is stored.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float to_tf32(float f)
{
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(f));
    return __uint_as_float(u);
}

// One entry of X split into hi + lo: TF32 parts in FP32 storage, or F16 parts
// of v scaled by xs (a power of two that puts X's largest entry near 2^14,
// undone exactly by the SYRK).  Returns whether either part is nonzero.
__device__ __forceinline__ bool store_x(void* Xh, void* Xl, size_t idx, float v, float xs, bool half)
{
    if (half) {
        const float vs = v * xs;
        const __half h = __float2half_rn(vs);
        const __half l = __float2half_rn(vs - __half2float(h));
        reinterpret_cast<__half*>(Xh)[idx] = h;
        reinterpret_cast<__half*>(Xl)[idx] = l;
        return __half2float(h) != 0.0f || __half2float(l) != 0.0f;
    }
    const float h = to_tf32(v);
    const float l = to_tf32(v - h);
    reinterpret_cast<float*>(Xh)[idx] = h;
    reinterpret_cast<float*>(Xl)[idx] = l;
    return h != 0.0f || l != 0.0f;
}

// column counts of the merged pre-PSF L, sqrt(C^-1) per active row, and the
// image pixel -> (active row, sqrt(C^-1)) table that k_psf_x reads: x fastest,
// with a border of half a PSF on every side so that no tap needs a bounds
// check (pixT[(j + pny/2) * (nx + 2 (pnx/2)) + i + pnx/2]; the rows of
// inactive and border pixels stay -1)
__global__ void k_csc_count(StaticData sd, const GridState* __restrict__ gs, const int* __restrict__ rowptr,
                            const int* __restrict__ cidx, const int* __restrict__ ccnt,
                            const double* __restrict__ cvec, const int* __restrict__ rowpix,
                            int* __restrict__ colcnt, float* __restrict__ sqc, int2* __restrict__ pixT)
{
    const int N = gs->N;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const int b = rowptr[r], n = ccnt[r];
        for (int e = 0; e < n; e++) atomicAdd(&colcnt[cidx[b + e]], 1);
        const float sq = sqrtf((float)cvec[r]);
        sqc[r] = sq;
        const int pix = rowpix[r];
        const int i = pix / sd.ny, j = pix - i * sd.ny;
        const int nxp = sd.nx + 2 * (sd.pnx / 2);
        pixT[(size_t)(j + sd.pny / 2) * nxp + i + sd.pnx / 2] = make_int2(r, __float_as_int(sq));
    }
}

// exclusive scan of colcnt[0..M) in place (colcnt[M] = total), cursor = starts
__global__ void __launch_bounds__(1024) k_csc_scan(const GridState* __restrict__ gs, int* __restrict__ colcnt,
                                                   int* __restrict__ cursor)
{
    __shared__ int part[1024];
    const int M = gs->M;
    const int per = (M + 1023) / 1024;
    const int a = threadIdx.x * per, b = min(a + per, M);
    int sum = 0;
    for (int i = a; i < b; i++) sum += colcnt[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {     // Hillis-Steele inclusive scan
        int v = (threadIdx.x >= off) ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - sum;
    for (int i = a; i < b; i++) {
        const int c = colcnt[i];
        colcnt[i] = run;
        cursor[i] = run;
        run += c;
    }
    if (threadIdx.x == 1023) colcnt[M] = part[1023];
}

__global__ void k_csc_fill(const GridState* __restrict__ gs, const int* __restrict__ rowptr,
                           const int* __restrict__ cidx, const int* __restrict__ ccnt, int* __restrict__ cursor,
                           int* __restrict__ col_u, int* __restrict__ src_u)
{
    const int N = gs->N;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const int b = rowptr[r], n = ccnt[r];
        for (int e = 0; e < n; e++) {
            const int pos = atomicAdd(&cursor[cidx[b + e]], 1);
            col_u[pos] = r;
            src_u[pos] = b + e;
        }
    }
}

// Each column's entries in increasing row order, so that every sum over a
// column runs in a fixed order (k_csc_fill places them in atomic order).
// Rows are distinct within a column of the merged L, so the order is a
// permutation: a bitonic sort of the (row, source position) pairs, a warp
// per column in registers for columns of up to CSC_SORT_WARP entries
// (k_csc_sort_w), else one CTA per column in shared memory for up to
// CSC_SORT_MAX entries, and past that each entry's rank counted directly.
#define CSC_SORT_MAX 4096
#define CSC_SORT_WARP 64    // columns sorted a warp each (k_csc_sort_w)
__global__ void __launch_bounds__(256) k_csc_sort(const GridState* __restrict__ gs, const int* __restrict__ colptr,
                                                  const int* __restrict__ col_u, const int* __restrict__ src_u,
                                                  const double* __restrict__ cval, int* __restrict__ colrow,
                                                  float* __restrict__ colval, double* __restrict__ colval64)
{
    __shared__ int key[CSC_SORT_MAX];
    __shared__ int pos[CSC_SORT_MAX];
    const int s = blockIdx.x;
    if (s >= gs->M) return;
    const int b = colptr[s], n = colptr[s + 1] - b;
    if (n <= CSC_SORT_WARP) return;                       // k_csc_sort_w's
    if (n <= CSC_SORT_MAX) {
        int p2 = 1;
        while (p2 < n) p2 <<= 1;
        for (int i = threadIdx.x; i < p2; i += blockDim.x) {
            key[i] = (i < n) ? col_u[b + i] : INT_MAX;
            pos[i] = (i < n) ? src_u[b + i] : 0;
        }
        __syncthreads();
        for (int k = 2; k <= p2; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = threadIdx.x; i < p2; i += blockDim.x) {
                    const int l = i ^ j;
                    if (l > i) {
                        const bool up = (i & k) == 0;
                        const int ki = key[i], kl = key[l];
                        if ((ki > kl) == up) {
                            key[i] = kl; key[l] = ki;
                            const int t = pos[i]; pos[i] = pos[l]; pos[l] = t;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double v = cval[pos[i]];
            colrow[b + i] = key[i];
            colval[b + i] = (float)v;
            colval64[b + i] = v;
        }
        return;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int ri = col_u[b + i];
        int rank = 0;
        for (int j = 0; j < n; j++) rank += (col_u[b + j] < ri) ? 1 : 0;
        const double v = cval[src_u[b + i]];
        colrow[b + rank] = ri;
        colval[b + rank] = (float)v;
        colval64[b + rank] = v;
    }
}

// Columns of up to CSC_SORT_WARP entries, a warp each: the same permutation
// by a bitonic network in registers (R = 1 or 2 entries a lane, entry
// lane + 32 h in register h; partners 32 apart within the lane, the others
// through lane shuffles; no barriers); k_csc_sort takes the longer columns
// (with more entries a lane the network's cost passed the block sort's).
// The rows are distinct, so any sort gives the same order.
__device__ __forceinline__ void csc_bitonic_step(int& key, int& pos, int e, int j, int k)
{
    const int kp = __shfl_xor_sync(0xffffffffu, key, j), pp = __shfl_xor_sync(0xffffffffu, pos, j);
    const bool up = ((e & ~j) & k) == 0;                  // the pair's direction, from its lower index
    const bool take_min = ((e & j) == 0) == up;
    if (take_min ? (kp < key) : (kp > key)) { key = kp; pos = pp; }
}

template <int R>
__device__ __forceinline__ void csc_sort_warp(const int* __restrict__ col_u, const int* __restrict__ src_u,
                                              const double* __restrict__ cval, int b, int n, int lane,
                                              int* __restrict__ colrow, float* __restrict__ colval,
                                              double* __restrict__ colval64)
{
    int key[R], pos[R];
    #pragma unroll
    for (int h = 0; h < R; h++) {
        const int e = lane + 32 * h;
        key[h] = (e < n) ? col_u[b + e] : INT_MAX;
        pos[h] = (e < n) ? src_u[b + e] : 0;
    }
    #pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
        #pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                #pragma unroll
                for (int h = 0; h < R; h++) {
                    const int h2 = h ^ (j >> 5);
                    if (h2 > h) {
                        const bool up = ((lane + 32 * h) & k) == 0;
                        if ((key[h] > key[h2]) == up) {
                            const int tk = key[h]; key[h] = key[h2]; key[h2] = tk;
                            const int tp = pos[h]; pos[h] = pos[h2]; pos[h2] = tp;
                        }
                    }
                }
            } else {
                #pragma unroll
                for (int h = 0; h < R; h++) csc_bitonic_step(key[h], pos[h], lane + 32 * h, j, k);
            }
        }
    }
    #pragma unroll
    for (int h = 0; h < R; h++) {
        const int e = lane + 32 * h;
        if (e < n) {
            const double v = cval[pos[h]];
            colrow[b + e] = key[h];
            colval[b + e] = (float)v;
            colval64[b + e] = v;
        }
    }
}

__global__ void __launch_bounds__(256, 4) k_csc_sort_w(const GridState* __restrict__ gs,
                                                       const int* __restrict__ colptr,
                                                       const int* __restrict__ col_u, const int* __restrict__ src_u,
                                                       const double* __restrict__ cval, int* __restrict__ colrow,
                                                       float* __restrict__ colval, double* __restrict__ colval64)
{
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= gs->M) return;                                // whole warps
    const int b = colptr[s], n = colptr[s + 1] - b;
    if (n <= 32) csc_sort_warp<1>(col_u, src_u, cval, b, n, lane, colrow, colval, colval64);
    else if (n <= CSC_SORT_WARP) csc_sort_warp<2>(col_u, src_u, cval, b, n, lane, colrow, colval, colval64);
}

// out[s] = sum over column s of L of value * w[row]: one warp per column, lane
// l takes entries l, l+32, ... in row order, then a fixed shuffle tree; zero
// from M up to the 64-padding.
__global__ void __launch_bounds__(256) k_LTw_csc(const GridState* __restrict__ gs, const int* __restrict__ colptr,
                                                 const int* __restrict__ colrow,
                                                 const double* __restrict__ colval64, const double* __restrict__ w,
                                                 double* __restrict__ out)
{
    const int M = gs->M, Mp = (M + 63) & ~63;
    const int lane = threadIdx.x & 31;
    for (int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); s < Mp; s += gridDim.x * (blockDim.x >> 5)) {
        double acc = 0;
        if (s < M) {
            const int b = colptr[s], e = colptr[s + 1];
            for (int k = b + lane; k < e; k += 32) acc += colval64[k] * w[colrow[k]];
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[s] = acc;
    }
}

// Schedule "bands": grid (M_cap cells, image-row bands).  Each CTA accumulates, for source cell
// s, the PSF-convolved image of column s of L on the image rows [j0, j1) of
// its band, in 64-bit fixed point on a dense shared-memory window that spans
// the bounding box of the footprints reaching the band (at most H rows x
// (nx + pnx - 1) columns), then writes X[s][r] = sqrt(C^-1)_r times that sum
// for every active pixel r of the band (zero outside the box).  The column's
// entries are sorted by active row, i.e. by image row j (j-outer order), so
// the entries that reach the band are one contiguous range, and so are the
// band's active rows; for each entry only the PSF rows that land in the band
// are visited, lanes along x (consecutive accumulators: the 64-bit shared
// atomics of one instruction do not collide).
__device__ __forceinline__ int lower_bound_row(const int* __restrict__ rowpix, const int* __restrict__ idx, int n,
                                               int ny, int jmin)
{
    // first position p in [0, n) whose pixel (rowpix[idx ? idx[p] : p]) has y index >= jmin
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int pix = rowpix[idx ? idx[mid] : mid];
        if (pix - (pix / ny) * ny < jmin) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// The same search by a whole warp (all lanes, converged): 32 probes per
// round narrow the range 32-fold, so a few rounds of dependent loads instead
// of log2(n).
__device__ __forceinline__ int warp_lower_bound_row(const int* __restrict__ rowpix, const int* __restrict__ idx,
                                                    int n, int ny, int jmin)
{
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = n;                       // the answer lies in [lo, hi]
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) / 32;
        const int p = lo + lane * step;
        bool ge = true;
        if (p < hi) {
            const int pix = rowpix[idx ? idx[p] : p];
            ge = pix - (pix / ny) * ny >= jmin;
        }
        const unsigned b = __ballot_sync(0xffffffffu, ge);
        if (b == 0) {
            lo = lo + 31 * step + 1;
        } else {
            const int f = __ffs(b) - 1;
            const int pf = lo + f * step;
            if (f > 0) lo = lo + (f - 1) * step + 1;
            hi = min(hi, pf);
        }
    }
    const int p = lo + lane;
    bool ge = true;
    if (p < hi) {
        const int pix = rowpix[idx ? idx[p] : p];
        ge = pix - (pix / ny) * ny >= jmin;
    }
    const unsigned b = __ballot_sync(0xffffffffu, ge);
    return b ? lo + __ffs(b) - 1 : hi;
}

// int64 -> float, rounded to nearest even, in integer arithmetic (the same
// result as the conversion instruction, which GB300 issues to its FP64 pipe):
// the top 24 significant bits, rounded on the bits below them.
__device__ __forceinline__ float ll2f_rn_int(long long v)
{
    if (v == 0) return 0.0f;
    const unsigned sign = v < 0 ? 0x80000000u : 0u;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    int e = 63 - __clzll((long long)a);          // index of the top bit
    unsigned m;
    if (e <= 23) {
        m = (unsigned)(a << (23 - e));
    } else {
        const int sh = e - 23;
        m = (unsigned)(a >> sh);
        const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (m & 1u))) {
            if (++m == (1u << 24)) { m >>= 1; e++; }
        }
    }
    return __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (m & 0x7fffffu));
}

// Eight consecutive entries of X (idx a multiple of 8): the F16 hi + lo
// parts as 16-byte stores (or the TF32 parts as 32-byte pairs).  Returns
// whether any part is nonzero.
__device__ __forceinline__ bool store_x8(void* Xh, void* Xl, size_t idx, const float* v, float xs, bool half)
{
    bool any = false;
    if (half) {
        __align__(16) __half h[8], l[8];
        #pragma unroll
        for (int u = 0; u < 8; u++) {
            const float vs = v[u] * xs;
            h[u] = __float2half_rn(vs);
            l[u] = __float2half_rn(vs - __half2float(h[u]));
            any |= __half2float(h[u]) != 0.0f || __half2float(l[u]) != 0.0f;
        }
        *reinterpret_cast<uint4*>(reinterpret_cast<__half*>(Xh) + idx) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(reinterpret_cast<__half*>(Xl) + idx) = *reinterpret_cast<const uint4*>(l);
        return any;
    }
    __align__(16) float h[8], l[8];
    #pragma unroll
    for (int u = 0; u < 8; u++) {
        h[u] = to_tf32(v[u]);
        l[u] = to_tf32(v[u] - h[u]);
        any |= h[u] != 0.0f || l[u] != 0.0f;
    }
    float4* ph = reinterpret_cast<float4*>(reinterpret_cast<float*>(Xh) + idx);
    float4* pl = reinterpret_cast<float4*>(reinterpret_cast<float*>(Xl) + idx);
    ph[0] = *reinterpret_cast<const float4*>(h);
    ph[1] = *reinterpret_cast<const float4*>(h + 4);
    pl[0] = *reinterpret_cast<const float4*>(l);
    pl[1] = *reinterpret_cast<const float4*>(l + 4);
    return any;
}

// Entries of a column staged in shared memory at a time by the band kernel
#define PSFX_ECHUNK 512

// The band schedule's per-item set-up, one warp per (source cell s, band):
// the range [e0, e1) of s's entries whose footprints reach the band's image
// rows [j0, j1), their bounding box and the window's image rows [wr0, wr1).
// meta[2 i] = (e0, e1, imin, imax), meta[2 i + 1] = (wr0, wr1, -, -) for
// item i = s * nband + band; an item without entries gets e0 = e1.
__global__ void __launch_bounds__(256) k_psfx_meta(StaticData sd, const GridState* __restrict__ gs,
                                                   const int* __restrict__ colptr, const int* __restrict__ colrow,
                                                   const int* __restrict__ rowpix, int H, int nband,
                                                   int4* __restrict__ meta)
{
    const int lane = threadIdx.x & 31;
    const int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int M = gs->M;
    const int Mp = (M + TC_TILE - 1) / TC_TILE * TC_TILE;
    const int s = item / nband, band = item - s * nband;
    if (s >= Mp) return;
    const int nyh = sd.pny / 2;
    const int j0 = band * H, j1 = min(j0 + H, sd.ny);
    const int b = (s < M) ? colptr[s] : 0, n = (s < M) ? colptr[s + 1] - b : 0;
    const int e0 = warp_lower_bound_row(rowpix, colrow + b, n, sd.ny, j0 - nyh);
    const int e1 = warp_lower_bound_row(rowpix, colrow + b, n, sd.ny, j1 + nyh);
    int4 m0 = make_int4(e0, e0, 0, 0), m1 = make_int4(j0, j0, 0, 0);
    if (e1 > e0) {
        int imn = INT_MAX, imx = INT_MIN, jmn = INT_MAX, jmx = INT_MIN;
        for (int e = e0 + lane; e < e1; e += 32) {
            const int pix = rowpix[colrow[b + e]];
            const int iq = pix / sd.ny, jq = pix - iq * sd.ny;
            imn = min(imn, iq); imx = max(imx, iq); jmn = min(jmn, jq); jmx = max(jmx, jq);
        }
        for (int o = 16; o > 0; o >>= 1) {
            imn = min(imn, __shfl_xor_sync(0xffffffffu, imn, o));
            imx = max(imx, __shfl_xor_sync(0xffffffffu, imx, o));
            jmn = min(jmn, __shfl_xor_sync(0xffffffffu, jmn, o));
            jmx = max(jmx, __shfl_xor_sync(0xffffffffu, jmx, o));
        }
        const int wr0 = max(j0, jmn - nyh), wr1 = min(j1, jmx - nyh + sd.pny);
        m0 = make_int4(e0, e1, imn, imx);
        m1 = make_int4(wr0, wr1, 0, 0);
    }
    if (lane == 0) {
        meta[2 * (size_t)item] = m0;
        meta[2 * (size_t)item + 1] = m1;
    }
}

// X's first Mp rows (cells) cleared by 16-byte stores, every column of X
// (K_cap, a multiple of 64): after the SYRK of the "rows" schedule, which
// writes every entry of its rows, so that X is all zero again for a band
// evaluation (whose own writes k_x_clean undoes).
__global__ void k_zero_x(const GridState* __restrict__ gs, uint4* __restrict__ Xh, uint4* __restrict__ Xl,
                         size_t row_vec)
{
    const int M = gs->M;
    const size_t n = (size_t)((M + TC_TILE - 1) / TC_TILE * TC_TILE) * row_vec;
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        Xh[i] = z;
        Xl[i] = z;
    }
}

// After the SYRK has read X: the entries the band kernel wrote (the active
// pixels of each item's window) set back to zero, so that X is all zero when
// the next evaluation's band kernel starts -- instead of clearing all of it
// (k_zero_x: ~480 MB per cfg5 evaluation) before.  The "rows" schedule
// writes every entry of its rows and clears X with k_zero_x after the SYRK.
__global__ void __launch_bounds__(256) k_x_clean(StaticData sd, const GridState* __restrict__ gs,
                                                 const int2* __restrict__ pixT, int nband,
                                                 const int4* __restrict__ meta, void* __restrict__ Xh,
                                                 void* __restrict__ Xl, int half, int K_cap)
{
    const int M = gs->M;
    const int Mp = (M + TC_TILE - 1) / TC_TILE * TC_TILE;
    const int s = blockIdx.x;
    if (s >= Mp) return;
    const size_t item = (size_t)s * nband + blockIdx.y;
    const int4 m0 = meta[2 * item], m1 = meta[2 * item + 1];
    if (m0.y <= m0.x) return;
    const int nxh = sd.pnx / 2, nyh = sd.pny / 2, nxp = sd.nx + 2 * nxh;
    const int imin = m0.z, Wb = m0.w - imin + sd.pnx, wr0 = m1.x, area = (m1.y - m1.x) * Wb;
    for (int e = threadIdx.x; e < area; e += blockDim.x) {
        const int jr = e / Wb, wc = e - jr * Wb;
        const int i = imin - nxh + wc, j = wr0 + jr;
        if (i < 0 || i >= sd.nx) continue;
        const int r = pixT[(size_t)(j + nyh) * nxp + i + nxh].x;
        if (r < 0) continue;
        const size_t idx = (size_t)s * K_cap + r;
        if (half) {
            reinterpret_cast<__half*>(Xh)[idx] = __float2half_rn(0.0f);
            reinterpret_cast<__half*>(Xl)[idx] = __float2half_rn(0.0f);
        } else {
            reinterpret_cast<float*>(Xh)[idx] = 0.0f;
            reinterpret_cast<float*>(Xl)[idx] = 0.0f;
        }
    }
}

// REGPSF (PSFs of at most 32 x 32 taps): lane pk holds PSF column pk in
// registers and an entry's footprint is visited row by row, fully unrolled
// -- no shared-memory loads of taps or offsets per tap, independent atomics
// back to back.  The integer sums are the same either way.
template <bool REGPSF>
__global__ void __launch_bounds__(512) k_psf_x_band(StaticData sd, const GridState* __restrict__ gs,
                                               const int* __restrict__ colptr, const int* __restrict__ colrow,
                                               const float* __restrict__ colval, const int* __restrict__ rowpix,
                                               const int2* __restrict__ pixT, int nband,
                                               const int4* __restrict__ meta, void* __restrict__ Xh,
                                               void* __restrict__ Xl, float xs, int half, int K_cap,
                                               unsigned char* __restrict__ nz, int nkb_cap)
{
    extern __shared__ __align__(16) unsigned char psfx_smem[];
    const int pnx = sd.pnx, pny = sd.pny, nxh = pnx / 2, nyh = pny / 2;
    const int nT = pnx * pny;
    const int M = gs->M;
    const int Mp = (M + TC_TILE - 1) / TC_TILE * TC_TILE;
    const int s = blockIdx.x;
    if (s >= Mp) return;
    const size_t item = (size_t)s * nband + blockIdx.y;
    const int4 m0 = meta[2 * item], m1 = meta[2 * item + 1];
    const int e0 = m0.x, e1 = m0.y, imin = m0.z;
    if (e1 <= e0) return;                                // nothing reaches the band: X stays zero
    const int wr0 = m1.x, wr1 = m1.y;
    const int Wb = m0.w - imin + pnx;                    // window columns imin - nxh .. imin - nxh + Wb - 1
    long long* acc = reinterpret_cast<long long*>(psfx_smem);
    int* tpsf = reinterpret_cast<int*>(acc + (size_t)(wr1 - wr0) * Wb);
    int* toff = tpsf + nT;
    int2* ent = reinterpret_cast<int2*>(toff + nT);      // staged entries (iq << 16 | jq, L): 8 nT bytes on, aligned
    const float inv = ldexpf(1.0f, -sd.fix_exp_x);
    const float lscale = ldexpf(1.0f, PSFX_LEXP);
    const int b = colptr[s];
    for (int i = threadIdx.x; i < (wr1 - wr0) * Wb; i += blockDim.x) acc[i] = 0;
    // taps in x-fastest order: tpsf[pl * pnx + pk] = psf[pk][pl] on its grid,
    // and the tap's offset in the window from the footprint's corner (the
    // register path reads the taps directly)
    if (!REGPSF) {
        for (int t = threadIdx.x; t < nT; t += blockDim.x) {
            const int pl = t / pnx, pk = t - pl * pnx;
            tpsf[t] = sd.psf_int[t];
            toff[t] = pl * Wb + pk;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int col[32];
    if (REGPSF) {
        #pragma unroll
        for (int pl = 0; pl < 32; pl++) col[pl] = (lane < pnx && pl < pny) ? sd.psf_int[pl * pnx + lane] : 0;
    }
    // the entries, PSFX_ECHUNK at a time: their pixel and L value staged in
    // shared memory by all threads (independent loads), then spread
    for (int c0 = e0; c0 < e1; c0 += PSFX_ECHUNK) {
        const int cn = min(PSFX_ECHUNK, e1 - c0);
        __syncthreads();
        for (int e = threadIdx.x; e < cn; e += blockDim.x) {
            const int pix = rowpix[colrow[b + c0 + e]];
            const int iq = pix / sd.ny, jq = pix - iq * sd.ny;
            ent[e] = make_int2((iq << 16) | jq, __float2int_rn(colval[b + c0 + e] * lscale));
        }
        __syncthreads();
        for (int e = warp; e < cn; e += nw) {
            const int2 en = ent[e];
            const int iq = en.x >> 16, jq = en.x & 0xffff;
            const int v = en.y;
            // PSF rows pl land on image row jq - nyh + pl; keep those in [wr0, wr1)
            const int pl0 = max(0, wr0 - (jq - nyh)), pl1 = min(pny, wr1 - (jq - nyh));
            if (REGPSF) {
                unsigned long long* cl = reinterpret_cast<unsigned long long*>(acc) + (jq - nyh - wr0) * Wb +
                                         (iq - imin) + lane;
                if (lane < pnx) {
                    #pragma unroll
                    for (int pl = 0; pl < 32; pl++)
                        if (pl >= pl0 && pl < pl1)
                            atomicAdd(cl + pl * Wb, (unsigned long long)((long long)col[pl] * (long long)v));
                }
            } else {
                // the footprint's corner (iq - nxh, jq - nyh) in window coordinates
                unsigned long long* corner =
                    reinterpret_cast<unsigned long long*>(acc) + (jq - nyh - wr0) * Wb + (iq - imin);
                const int t1 = pl1 * pnx;
                for (int t = pl0 * pnx + lane; t < t1; t += 32)
                    atomicAdd(corner + toff[t], (unsigned long long)((long long)tpsf[t] * (long long)v));
            }
        }
    }
    __syncthreads();
    // X[s][r] for the active pixels r of the window: v = sqrt(C^-1)_r * sum,
    // split into hi + lo; the window's pixels are visited x fastest through
    // the padded image's (active row, sqrt(C^-1)) table.  Every other entry
    // of X's row s is zero (X is all zero between evaluations: k_x_clean).
    {
        const int nxp = sd.nx + 2 * nxh;
        const int area = (wr1 - wr0) * Wb;
        for (int e = threadIdx.x; e < area; e += blockDim.x) {
            const int jr = e / Wb, wc = e - jr * Wb;
            const int i = imin - nxh + wc, j = wr0 + jr;
            if (i < 0 || i >= sd.nx) continue;
            const int2 pt = pixT[(size_t)(j + nyh) * nxp + i + nxh];
            if (pt.x < 0) continue;
            const float v = (ll2f_rn_int(acc[e]) * inv) * __int_as_float(pt.y);
            if (store_x(Xh, Xl, (size_t)s * K_cap + pt.x, v, xs, half))
                nz[(size_t)(s / TC_TILE) * nkb_cap + pt.x / TC_KB] = 1;
        }
    }
}

// Schedule "rows": grid (M_cap cells, chunks of active rows); one CTA holds
// the 64-bit accumulators of a chunk of active rows and scatters each entry
// of column s over its PSF footprint through the active-row table of the
// padded image (pixT).  Each product psf x L is the same exact integer
// product and sqrt(C^-1) is applied to the sum as in the "bands" schedule, so
// both give the same bits.
__global__ void __launch_bounds__(512) k_psf_x_rows(StaticData sd, const GridState* __restrict__ gs,
                                               const int* __restrict__ colptr, const int* __restrict__ colrow,
                                               const float* __restrict__ colval, const int* __restrict__ rowpix,
                                               const int2* __restrict__ pixT, const float* __restrict__ sqc,
                                               int chunk, void* __restrict__ Xh, void* __restrict__ Xl, float xs,
                                               int half, int K_cap, unsigned char* __restrict__ nz,
                                               int nkb_cap)
{
    extern __shared__ __align__(16) unsigned char psfx_smem[];
    long long* acc = reinterpret_cast<long long*>(psfx_smem);
    int* tpsf = reinterpret_cast<int*>(acc + chunk);
    const int N = gs->N, M = gs->M;
    const int Mp = (M + TC_TILE - 1) / TC_TILE * TC_TILE;
    const int Np = (N + 63) & ~63;                           // whole 64-pixel stages for the F16 SYRK
    const int s = blockIdx.x;
    const int r0 = blockIdx.y * chunk, r1 = min(r0 + chunk, Np);
    if (s >= Mp || r0 >= Np) return;
    const int nT = sd.pnx * sd.pny;
    const float inv = ldexpf(1.0f, -sd.fix_exp_x);
    const int pnx = sd.pnx;
    const int nxp = sd.nx + 2 * (pnx / 2);                    // padded width of pixT
    int* toff = reinterpret_cast<int*>(tpsf + nT);
    for (int i = threadIdx.x; i < r1 - r0; i += blockDim.x) acc[i] = 0;
    // taps in x-fastest order: tpsf[pl * pnx + pk] = psf[pk][pl] on its grid
    // (StaticData::psf_int), and the tap's offset in pixT from the
    // footprint's corner
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        const int pl = t / pnx, pk = t - pl * pnx;
        tpsf[t] = sd.psf_int[t];
        toff[t] = pl * nxp + pk;
    }
    const float lscale = ldexpf(1.0f, PSFX_LEXP);
    __syncthreads();
    if (s < M) {
        const int b = colptr[s], n = colptr[s + 1] - b;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int e = warp; e < n; e += nw) {
            const int q = colrow[b + e];
            const long long v = __float2int_rn(colval[b + e] * lscale);     // L on its grid
            const int pix = rowpix[q];
            const int iq = pix / sd.ny, jq = pix - iq * sd.ny;
            // the footprint's corner (iq - pnx/2, jq - pny/2) sits at (iq, jq) of
            // the padded table; lanes run along x, so the targets of one
            // instruction are consecutive active rows and its 64-bit shared
            // atomics do not collide
            const int2* corner = pixT + (size_t)jq * nxp + iq;
            // four taps per lane in flight: their table loads are independent
            for (int t0 = lane; t0 < nT; t0 += 128) {
                int2 P[4];
                int w[4];
                #pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int t = t0 + 32 * u;
                    P[u] = make_int2(-1, 0);
                    w[u] = 0;
                    if (t < nT) {
                        P[u] = corner[toff[t]];
                        w[u] = tpsf[t];
                    }
                }
                #pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (P[u].x >= r0 && P[u].x < r1)                // inactive (-1) or another chunk
                        atomicAdd(reinterpret_cast<unsigned long long*>(&acc[P[u].x - r0]),
                                  (unsigned long long)((long long)w[u] * v));
                }
            }
        }
    }
    __syncthreads();
    // write row s of X for pixels [r0, r1): v = sqrt(C^-1)_r * sum split into
    // hi + lo (zero beyond the N active rows); one warp covers one 32-pixel block
    const int span = r1 - r0;
    for (int i0 = 0; i0 < span; i0 += blockDim.x) {
        const int i = i0 + threadIdx.x;
        bool nonzero = false;
        if (i < span) {
            const float v = (r0 + i < N) ? (ll2f_rn_int(acc[i]) * inv) * sqc[r0 + i] : 0.0f;
            nonzero = store_x(Xh, Xl, (size_t)s * K_cap + r0 + i, v, xs, half);
        }
        const unsigned any = __ballot_sync(0xffffffffu, nonzero);
        if ((threadIdx.x & 31) == 0 && any && i < span)
            nz[(size_t)(s / TC_TILE) * nkb_cap + (r0 + i) / TC_KB] = 1;
    }
}

// F32 += lambda R; R32 = R; identity beyond M up to the 64-padding.
__device__ __forceinline__ int act_at32(const int* ai, int snx, int sny, int i, int j)
{
    if (i < 0 || j < 0 || i >= snx || j >= sny) return -1;
    return ai[j * snx + i];
}

__global__ void k_reg32(const GridState* __restrict__ gs, const int* __restrict__ ai,
                        const double* __restrict__ regp, float* __restrict__ F, float* __restrict__ R, int ld,
                        int do_reg, int parts)
{
    const bool toF = parts & REG_F, toR = parts & REG_R;
    const double regparam = *regp;
    const int snx = gs->snx, sny = gs->sny;
    const int M = gs->M, Mp = (M + 127) & ~127;   // identity up to the 128-block padding
    const int ncell = snx * sny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell + (Mp - M); c += gridDim.x * blockDim.x) {
        if (c >= ncell) {
            int i = M + (c - ncell);
            if (toF) F[(size_t)i * ld + i] = 1.0f;
            if (do_reg && toR) R[(size_t)i * ld + i] = 1.0f;
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
        if (toR) R[(size_t)a * ld + a] = (float)diag;
        if (toF) F[(size_t)a * ld + a] = (float)((double)F[(size_t)a * ld + a] + regparam * diag);
        for (int k = 0; k < 4; k++) {
            int b = nb1[k];
            if (b >= 0 && b < a) {
                if (toR) R[(size_t)a * ld + b] = -4.0f;
                if (toF) F[(size_t)a * ld + b] = (float)((double)F[(size_t)a * ld + b] - 4.0 * regparam);
            }
            int b2 = nb2[k];
            if (b2 >= 0 && nb1[k] >= 0 && b2 < a) {
                if (toR) R[(size_t)a * ld + b2] = 1.0f;
                if (toF) F[(size_t)a * ld + b2] = (float)((double)F[(size_t)a * ld + b2] + regparam);
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
                           const double* __restrict__ vv, const int* __restrict__ ai,
                           const double* __restrict__ regp, int do_reg, const double* __restrict__ s,
                           double* __restrict__ r)
{
    const double regparam = *regp;
    const int snx = gs->snx, sny = gs->sny;
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
    void* ptrs[] = {m->t, m->X_hi, m->X_lo, m->nz, m->F32, m->R32, m->u, m->v, m->r, m->z, m->y, m->img,
                    m->linvF, m->linv128, m->yf, m->zf, m->flags, m->colcnt, m->cursor, m->colrow, m->colval,
                    m->sqc, m->col_u, m->src_u, m->colval64, m->pixT, m->F0, m->Pf_hi, m->Pf_lo, m->Pf_exp,
                    m->Pr_hi, m->Pr_lo, m->Pr_exp, m->psfx_meta};
    for (void* p : ptrs) if (p) cudaFree(p);
    delete m;
    c.mixed = nullptr;
}

// The band schedule's geometry: image rows per band H -- as many as fit
// beside the PSF tables in about half an SM's shared memory (two CTAs per
// SM), divided by `split` -- the number of bands and the dynamic shared
// memory of a CTA.
static void psfx_band_geom(int nx, int ny, int pnx, int pny, int split, int& H, int& nband, size_t& smem)
{
    const int nT = pnx * pny;
    const int W = nx + pnx - 1;
    const size_t tap_bytes = 2 * sizeof(int) * (size_t)nT + 8 * sizeof(int) + 2 * sizeof(int) * PSFX_ECHUNK;
    const size_t avail = (110 * 1024 > tap_bytes) ? 110 * 1024 - tap_bytes : 0;
    const int fit = std::max(1, (int)(avail / (sizeof(long long) * W)));
    H = std::max(1, std::min(ny, fit) / split);
    nband = (ny + H - 1) / H;
    smem = sizeof(long long) * (size_t)H * W + tap_bytes;
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
    const size_t xbytes = (m->half ? 2 : 4) * (size_t)M_cap * K_cap;
    A((void**)&m->X_hi, xbytes);
    A((void**)&m->X_lo, xbytes);
    A((void**)&m->nz, (size_t)(M_cap / TC_TILE) * m->nkb_cap);
    {
        int H = 1;
        size_t sm = 0;
        psfx_band_geom(c.img_nx, c.img_ny, c.psf_nx, c.psf_ny, 4, H, m->psfx_bands, sm);   // the finest split
        A((void**)&m->psfx_meta, sizeof(int4) * 2 * (size_t)M_cap * m->psfx_bands);
    }
    A((void**)&m->F32, sizeof(float) * (size_t)M_cap * M_cap);
    A((void**)&m->R32, sizeof(float) * (size_t)M_cap * M_cap);
    m->nnz_cap = 3 * c.N_cap * c.nsub_cap;
    A((void**)&m->colcnt, sizeof(int) * (size_t)(M_cap + 1));
    A((void**)&m->cursor, sizeof(int) * (size_t)M_cap);
    A((void**)&m->colrow, sizeof(int) * (size_t)m->nnz_cap);
    A((void**)&m->colval, sizeof(float) * (size_t)m->nnz_cap);
    A((void**)&m->col_u, sizeof(int) * (size_t)m->nnz_cap);
    A((void**)&m->pixT, sizeof(int2) * (size_t)c.npix_pad);
    A((void**)&m->img, sizeof(double) * (size_t)c.npix_pad);
    A((void**)&m->src_u, sizeof(int) * (size_t)m->nnz_cap);
    A((void**)&m->colval64, sizeof(double) * (size_t)m->nnz_cap);
    A((void**)&m->sqc, sizeof(float) * (size_t)(c.N_cap + 64));
    A((void**)&m->t, sizeof(double) * (size_t)(c.N_cap + 64));
    A((void**)&m->u, sizeof(double) * (size_t)(c.N_cap + 64));
    A((void**)&m->v, sizeof(double) * M_cap);
    A((void**)&m->r, sizeof(double) * M_cap);
    A((void**)&m->z, sizeof(double) * M_cap);
    A((void**)&m->y, sizeof(double) * M_cap);
    m->nb = M_cap / C2;
    A((void**)&m->linvF, sizeof(float) * (size_t)m->nb * 2 * C2 * C2);
    A((void**)&m->linv128, sizeof(float) * 2 * C2 * C2);
    A((void**)&m->yf, sizeof(float) * (size_t)M_cap);
    A((void**)&m->zf, sizeof(float) * (size_t)M_cap);
    A((void**)&m->flags, sizeof(int) * (size_t)2 * m->nb);
    A((void**)&m->Pf_hi, sizeof(__half) * (size_t)M_cap * C2);
    A((void**)&m->Pf_lo, sizeof(__half) * (size_t)M_cap * C2);
    A((void**)&m->Pr_hi, sizeof(__half) * (size_t)M_cap * C2);
    A((void**)&m->Pr_lo, sizeof(__half) * (size_t)M_cap * C2);
    A((void**)&m->Pf_exp, sizeof(int) * (size_t)M_cap);
    A((void**)&m->Pr_exp, sizeof(int) * (size_t)M_cap);
    if (e != cudaSuccess) {
        set_error("%s (%d)", "mixed-precision workspace allocation failed", (int)e);
        return QLP_ERR_NOMEM;
    }
    cudaMemset(m->X_hi, 0, xbytes);
    cudaMemset(m->X_lo, 0, xbytes);
    if (make_map(&m->map_hi, m->X_hi, M_cap, K_cap, m->half) != QLP_OK ||
        make_map(&m->map_lo, m->X_lo, M_cap, K_cap, m->half) != QLP_OK ||
        make_map(&m->map_pf_hi, m->Pf_hi, M_cap, C2, true) != QLP_OK ||
        make_map(&m->map_pf_lo, m->Pf_lo, M_cap, C2, true) != QLP_OK ||
        make_map(&m->map_pr_hi, m->Pr_hi, M_cap, C2, true) != QLP_OK ||
        make_map(&m->map_pr_lo, m->Pr_lo, M_cap, C2, true) != QLP_OK) {
        set_error("%s (%d)", "cuTensorMapEncodeTiled unavailable or failed", 0);
        return QLP_ERR_CUDA;
    }
    // shared-memory opt-ins (a kernel's static and dynamic shared memory
    // together may not pass 227 KB): a failed opt-in is reported here, not at
    // the first launch that needs it
    {
        cudaError_t ea = cudaSuccess;
        auto opt = [&](const void* f, int bytes) {
            const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (ea == cudaSuccess) ea = r;
        };
        opt((const void*)k_psf_x_rows, 227 * 1024);
        opt((const void*)k_psf_x_band<true>, 227 * 1024);
        opt((const void*)k_psf_x_band<false>, 227 * 1024);
        opt((const void*)k_potrf128, P128_SMEM);
        opt((const void*)k_chol_tile128, T128_SMEM);
        opt((const void*)k_chol_upd16, U16_SMEM);
        opt((const void*)k_syrk_tc<false>, TC_SMEM);
        opt((const void*)k_syrk_tc<true>, TC_SMEM);
        if (ea != cudaSuccess) {
            set_error("%s (%d)", "shared-memory opt-in failed", (int)ea);
            return QLP_ERR_CUDA;
        }
    }
    m->ready = true;
    return QLP_OK;
}

// FP32 blocked Cholesky for the mixed path (chol128.cuh): per 128-column step
// the diagonal factor and its inverse in one CTA, the panel solve on the
// tensor cores (which also leaves the panel split into F16 hi + lo in
// P_hi / P_lo, addressed by map_hi / map_lo), and the trailing update from
// that split panel on the tensor cores.  band: 128-blocks below the diagonal
// that can be nonzero (the whole matrix for F).  The inverse of diagonal
// block k goes to linv + k * linv_stride (stride 0: one scratch block).
static int cholesky_mixed(float* A, int ld, int M_cap128, GridState* gs, int which, int band, float* linv,
                          size_t linv_stride, __half* P_hi, __half* P_lo, int* pexp, const CUtensorMap& map_hi,
                          const CUtensorMap& map_lo, cudaStream_t st)
{
    const int nb = M_cap128 / C2;
    int n = 0;
    for (int k = 0; k < nb; k++) {
        float* lk = linv + (size_t)k * linv_stride;
        k_potrf128<<<1, 256, P128_SMEM, st>>>(A, ld, k, gs, which, lk);
        n++;
        const int rem = nb - k - 1;
        if (rem == 0) break;
        const int bt = std::min(rem, band);
        k_chol_tile128<<<bt, 128, T128_SMEM, st>>>(A, ld, k, gs, 1, lk, band, P_hi, P_lo, pexp);
        k_chol_upd16<<<bt * (bt + 1) / 2, 128, U16_SMEM, st>>>(map_hi, map_lo, A, ld, k, gs, pexp, band);
        n += 2;
    }
    count_launches(n);
    return n;
}

// The lambda optimisation's F0 = X X^T (before lambda R): allocated outside
// any stream capture, before the first PIPE_PRE / PIPE_TRIAL sequence.
int mixed_ensure_f0(Slot& slot)
{
    int rc = mixed_init(slot);
    if (rc != QLP_OK) return rc;
    MixedWork* m = mw_of(slot);
    if (m->F0) return QLP_OK;
    if (cudaMalloc(&m->F0, sizeof(float) * (size_t)m->ld32 * m->M_cap) != cudaSuccess) {
        m->F0 = nullptr;
        set_error("%s (%d)", "lambda optimisation workspace allocation failed", m->M_cap);
        return QLP_ERR_NOMEM;
    }
    return QLP_OK;
}

// part: PIPE_ALL the whole inversion at the slot's lambda; PIPE_PRE everything
// that does not depend on lambda (D, X, F0 = X X^T kept aside, R and its log
// det); PIPE_TRIAL one lambda of the optimisation (F = F0 + lambda R, its
// factor, log det and the refined amplitudes, the model image).
int run_inversion_mixed(const qlp_ctx* c, Slot& slot, const StaticData& sd, const SrcOpts& so, const double* regp,
                        int part, cudaStream_t st, cudaEvent_t* ev)
{
    const int refine = c->refine;
    int rc = mixed_init(slot);
    if (rc != QLP_OK) return rc;
    MixedWork* m = mw_of(slot);
    Work& w = slot.w;
    const int N_cap = sd.n_mask;
    const int Mc = slot.M_cap;
    const size_t f_bytes = sizeof(float) * (size_t)m->ld32 * m->M_cap;
    const int ltw_blocks = (m->M_cap + 7) / 8;
    int n = 0;
    if (part != PIPE_ALL && !m->F0) {
        set_error("%s (%d)", "lambda optimisation workspace missing", part);
        return QLP_ERR_ARG;
    }
    if (part == PIPE_TRIAL) {
        cudaMemsetAsync(&w.gs->not_spd_F, 0, sizeof(int), st);
        cudaMemcpyAsync(m->F32, m->F0, f_bytes, cudaMemcpyDeviceToDevice, st);
        k_reg32<<<(so.snx * so.sny + 128 + 255) / 256, 256, 0, st>>>(w.gs, w.active_index, regp, m->F32, m->R32,
                                                                    m->ld32, so.regularization, REG_F);
        n++;
    } else {

    // L by source cell (CSC, rows ascending within a column)
    cudaMemsetAsync(m->nz, 0, (size_t)(m->M_cap / TC_TILE) * m->nkb_cap, st);
    cudaMemsetAsync(m->colcnt, 0, sizeof(int) * (size_t)(m->M_cap + 1), st);
    {
        const int rb = std::min((N_cap + 255) / 256, 152 * 8);
        cudaMemsetAsync(m->pixT, 0xff, sizeof(int2) * (size_t)slot.npix_pad, st);
        k_csc_count<<<std::max(rb, 1), 256, 0, st>>>(sd, w.gs, w.rowptr, w.cidx, w.ccnt, w.cvec, w.rowpix, m->colcnt,
                                                     m->sqc, m->pixT);
        k_csc_scan<<<1, 1024, 0, st>>>(w.gs, m->colcnt, m->cursor);
        k_csc_fill<<<std::max(rb, 1), 256, 0, st>>>(w.gs, w.rowptr, w.cidx, w.ccnt, m->cursor, m->col_u, m->src_u);
        k_csc_sort_w<<<(m->M_cap + 7) / 8, 256, 0, st>>>(w.gs, m->colcnt, m->col_u, m->src_u, w.cval, m->colrow,
                                                        m->colval, m->colval64);
        k_csc_sort<<<m->M_cap, 256, 0, st>>>(w.gs, m->colcnt, m->col_u, m->src_u, w.cval, m->colrow, m->colval,
                                            m->colval64);
        n += 5;
    }
    // D = L^T P^T (C^-1 d), FP64
    op_conv(sd, w, N_cap, true, w.dvec, w.cvec, m->t, m->img, m->pixT, st);
    k_LTw_csc<<<ltw_blocks, 256, 0, st>>>(w.gs, m->colcnt, m->colrow, m->colval64, m->t, w.D);
    n++;
    // X = (P L sqrt(C^-1))^T and its block flags, from L by source cell
    const float xs = m->half ? ldexpf(1.0f, sd.x_exp) : 1.0f;     // F16 scale of X
    int band_nband = 0;                                               // bands of the band schedule (0: rows)
    {
        const int nT = sd.pnx * sd.pny;
        const int split = std::max(1, std::min(c->psfx_split, 4));
        const int pt = (c->psfx_threads == 128 || c->psfx_threads == 512) ? c->psfx_threads : 256;
        if (c->psfx_mode == 1) {
            int H = 1, nband = 1;
            size_t smem = 0;
            psfx_band_geom(sd.nx, sd.ny, sd.pnx, sd.pny, split, H, nband, smem);
            // each item's set-up, then the windows (X is all zero here: the
            // previous evaluation cleaned it after its SYRK, see below)
            band_nband = nband;
            k_psfx_meta<<<(m->M_cap * nband + 7) / 8, 256, 0, st>>>(sd, w.gs, m->colcnt, m->colrow, w.rowpix, H,
                                                                  nband, m->psfx_meta);
            if (sd.pnx <= 32 && sd.pny <= 32)
                k_psf_x_band<true><<<dim3(m->M_cap, nband), pt, smem, st>>>(
                    sd, w.gs, m->colcnt, m->colrow, m->colval, w.rowpix, m->pixT, nband, m->psfx_meta, m->X_hi,
                    m->X_lo, xs, m->half ? 1 : 0, m->K_cap, m->nz, m->nkb_cap);
            else
                k_psf_x_band<false><<<dim3(m->M_cap, nband), pt, smem, st>>>(
                    sd, w.gs, m->colcnt, m->colrow, m->colval, w.rowpix, m->pixT, nband, m->psfx_meta, m->X_hi,
                    m->X_lo, xs, m->half ? 1 : 0, m->K_cap, m->nz, m->nkb_cap);
            n += 1;
        } else {
            // accumulator rows per CTA: the active rows split into psfx_split
            // chunks (or more, if a chunk does not fit beside the PSF in 227 KB)
            const int fit = (int)(((227 * 1024 - (sizeof(float) + sizeof(int)) * (size_t)nT) / sizeof(long long)) &
                                  ~(size_t)31);
            const int want = ((m->K_cap + split - 1) / split + 31) & ~31;
            const int chunk = std::max(32, std::min(want, fit));
            const int nchunk = (m->K_cap + chunk - 1) / chunk;
            const size_t smem = sizeof(long long) * (size_t)chunk + (sizeof(float) + sizeof(int)) * (size_t)nT;
            k_psf_x_rows<<<dim3(m->M_cap, nchunk), pt, smem, st>>>(sd, w.gs, m->colcnt, m->colrow, m->colval,
                                                                    w.rowpix, m->pixT, m->sqc, chunk, m->X_hi,
                                                                    m->X_lo, xs, m->half ? 1 : 0, m->K_cap, m->nz,
                                                                    m->nkb_cap);
        }
        n++;
    }
    if (ev) cudaEventRecord(ev[3], st);
    {
        const int nt = m->M_cap / TC_TILE;
        if (m->half)
            k_syrk_tc<true><<<nt * (nt + 1) / 2, 128, TC_SMEM, st>>>(m->map_hi, m->map_lo, w.gs, m->nz, m->nkb_cap,
                                                                      m->F32, m->ld32, ldexpf(1.0f, -2 * sd.x_exp));
        else
            k_syrk_tc<false><<<nt * (nt + 1) / 2, 128, TC_SMEM, st>>>(m->map_hi, m->map_lo, w.gs, m->nz,
                                                                       m->nkb_cap, m->F32, m->ld32, 1.0f);
        n++;
        // X back to all zero for the next evaluation
        if (band_nband > 0) {
            k_x_clean<<<dim3(m->M_cap, band_nband), 256, 0, st>>>(sd, w.gs, m->pixT, band_nband, m->psfx_meta,
                                                                  m->X_hi, m->X_lo, m->half ? 1 : 0, m->K_cap);
        } else {
            const size_t row_vec = (size_t)m->K_cap * (m->half ? 2 : 4) / 16;
            k_zero_x<<<152 * 8, 256, 0, st>>>(w.gs, reinterpret_cast<uint4*>(m->X_hi),
                                              reinterpret_cast<uint4*>(m->X_lo), row_vec);
        }
        n++;
    }
    if (ev) cudaEventRecord(ev[4], st);
    if (part == PIPE_PRE) cudaMemcpyAsync(m->F0, m->F32, f_bytes, cudaMemcpyDeviceToDevice, st);
    if (so.regularization) cudaMemsetAsync(m->R32, 0, sizeof(float) * (size_t)m->ld32 * m->ld32, st);
    k_reg32<<<(so.snx * so.sny + 128 + 255) / 256, 256, 0, st>>>(w.gs, w.active_index, regp, m->F32, m->R32,
                                                                m->ld32, so.regularization,
                                                                part == PIPE_PRE ? REG_R : (REG_F | REG_R));
    n++;
    if (so.regularization) {
        // R's factorisation (log det R only) runs on the slot's second stream,
        // beside F's.  R couples a cell to cells at most two grid rows
        // (2 snx active indices) away, so its factor stays within that band.
        cudaEventRecord(slot.side_fork, st);
        cudaStreamWaitEvent(slot.side, slot.side_fork, 0);
        const int band_R = (2 * so.snx - 1) / C2 + 1;
        n += cholesky_mixed(m->R32, m->ld32, m->M_cap, w.gs, 1, band_R, m->linv128, 0, m->Pr_hi, m->Pr_lo,
                            m->Pr_exp, m->map_pr_hi, m->map_pr_lo, slot.side);
        k_logdet_t<float><<<1, 1024, 0, slot.side>>>(m->R32, m->ld32, w.gs, w.out, 1);
        n++;
        cudaEventRecord(slot.side_join, slot.side);
    }
    if (part == PIPE_PRE) {
        if (so.regularization) cudaStreamWaitEvent(st, slot.side_join, 0);
        count_launches(n);
        return QLP_OK;
    }
    }   // part != PIPE_TRIAL
    n += cholesky_mixed(m->F32, m->ld32, m->M_cap, w.gs, 0, 1 << 20, m->linvF, (size_t)2 * C2 * C2, m->Pf_hi,
                        m->Pf_lo, m->Pf_exp, m->map_pf_hi, m->map_pf_lo, st);
    k_logdet_t<float><<<1, 1024, 0, st>>>(m->F32, m->ld32, w.gs, w.out, 0);
    n++;
    if (so.regularization && part == PIPE_ALL) cudaStreamWaitEvent(st, slot.side_join, 0);
    // s = F^-1 D with `refine` FP64 refinement sweeps
    k_copy_init<<<(Mc + 255) / 256, 256, 0, st>>>(w.gs, w.D, m->r, w.s);
    n++;
    for (int it = 0; it <= refine; it++) {
        cudaMemsetAsync(m->flags, 0, sizeof(int) * (size_t)2 * m->nb, st);
        k_trsv128_fwd<<<m->nb, 256, 0, st>>>(m->F32, m->ld32, m->linvF, w.gs, m->r, m->yf, m->flags);
        k_trsv128_bwd<<<m->nb, 256, 0, st>>>(m->F32, m->ld32, m->linvF, w.gs, m->yf, m->zf, m->z,
                                              m->flags + m->nb);
        k_axpy<<<(Mc + 255) / 256, 256, 0, st>>>(w.gs, m->z, w.s);
        n += 3;
        if (it == refine) break;
        op_Ls(w, N_cap, w.s, m->t, st);
        op_conv(sd, w, N_cap, false, m->t, nullptr, m->u, m->img, m->pixT, st);
        op_conv(sd, w, N_cap, true, m->u, w.cvec, m->t, m->img, m->pixT, st);
        k_LTw_csc<<<ltw_blocks, 256, 0, st>>>(w.gs, m->colcnt, m->colrow, m->colval64, m->t, m->v);
        n++;
        k_residual<<<(so.snx * so.sny + 255) / 256, 256, 0, st>>>(w.gs, w.D, m->v, w.active_index, regp,
                                                                  so.regularization, w.s, m->r);
        n++;
    }
    // model image P L s in FP64 for chi^2
    op_Ls(w, N_cap, w.s, m->t, st);
    op_conv(sd, w, N_cap, false, m->t, nullptr, w.model, m->img, m->pixT, st);
    count_launches(n);
    return QLP_OK;
}

}  // namespace qlpix
