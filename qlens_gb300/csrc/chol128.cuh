// chol128.cuh -- FP32 blocked Cholesky with 128-wide steps for the mixed path.
//
// Right-looking, one 128-column block per step k:
//   k_potrf128       one CTA factors the 128x128 diagonal block in shared
//                    memory (four 32-column panels: a warp factors the 32x32
//                    diagonal piece in registers, the rows below are solved
//                    one per thread, the trailing piece is updated with 4x4
//                    register blocks) and inverts the factor (diagonal 32x32
//                    inverses by forward substitution, off-diagonal blocks by
//                    V_ij = -V_ii sum_k L_ik V_kj);
//   k_chol_tile128   mode 1 (panel solve): P_I <- P_I L_kk^-T for the 128-row
//                    blocks below, as 128x128x128 products on the tensor cores
//                    (tcgen05 kind::tf32, 3xTF32 split, accumulator in TMEM),
//                    K in four quarters of 32; its epilogue also writes each
//                    solved block once as F16 hi + lo, each row scaled by a
//                    power of two (its largest entry near 2^14), into the
//                    panel buffer;
//   k_chol_upd16     the trailing update A_IJ -= P_I P_J^T for the
//                    lower-triangle tiles: TMA loads of the split panel
//                    blocks (128-byte swizzle), tcgen05 kind::f16 at twice
//                    the TF32 rate, three products (hi*hi + hi*lo + lo*hi,
//                    ~22 significant bits), the scales undone in the
//                    epilogue.  (mode 0 of k_chol_tile128 computes the same
//                    update from the FP32 panel, re-split per tile.)
// `band` limits both to the tiles within that many 128-blocks of the
// diagonal: the curvature matrix R couples a cell only to cells at most two
// grid rows away, so its factor stays inside that band (dense F passes a
// band larger than the matrix).
// QLens factors with Cholesky_dcmp_packed (pixelgrid.cpp:17071-17105): a
// negative pivot is recorded and sqrt(|d|) used; the first such pivot is
// reported through GridState::not_spd_F / not_spd_R.
#pragma once
#include <cuda_fp16.h>
#include "tc_common.cuh"

namespace qlpix {

#define C2 128
#define P128_SMEM (2 * C2 * (C2 + 1) * 4 + 32 * 33 * 4 + C2 * 4)         // S, V, T, 1/diag
#define T128_SMEM (4 * TC_TILE_BYTES + 1024)                             // [A/B][hi/lo], one K quarter
#define U16_SMEM (4 * TC_TILE_BYTES + 1024)                              // [A/B][hi/lo], one K half (64 F16)

__device__ __forceinline__ int cpad128(int M) { return (M + C2 - 1) / C2 * C2; }

__device__ __forceinline__ void tri_ij(int t, int& i, int& j)
{
    i = (int)((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);   // corrected below
    while ((i + 1) * (i + 2) / 2 <= t) i++;
    while (i * (i + 1) / 2 > t) i--;
    j = t - i * (i + 1) / 2;
}

// One step of the register Cholesky of a 32x32 block held one row per lane
// (lane l: a[c] = L[l][c]); unrolled at compile time so a[] stays in registers.
template <int J>
__device__ __forceinline__ void warp_chol32(float (&a)[32], int lane, int* flag, int pivot0)
{
    if constexpr (J < 32) {
        const float d = __shfl_sync(0xffffffffu, a[J], J);
        if (lane == 0 && d < 0.f && *flag == 0) *flag = pivot0 + J + 1;
        const float rs = rsqrtf(fabsf(d));      // FP32 path: 1/sqrt and a multiply, not sqrt and a divide
        if (lane == J) a[J] = fabsf(d) * rs;
        else if (lane > J) a[J] = a[J] * rs;
        #pragma unroll
        for (int c = J + 1; c < 32; c++) {
            const float vc = __shfl_sync(0xffffffffu, a[J], c);
            if (lane >= c) a[c] -= a[J] * vc;
        }
        warp_chol32<J + 1>(a, lane, flag, pivot0);
    }
}

__global__ void __launch_bounds__(256, 1) k_potrf128(float* __restrict__ A, int ld, int k, GridState* gs, int which,
                                                  float* __restrict__ Linv)
{
    extern __shared__ float p128_smem[];
    float (*S)[C2 + 1] = reinterpret_cast<float (*)[C2 + 1]>(p128_smem);
    float (*V)[C2 + 1] = reinterpret_cast<float (*)[C2 + 1]>(p128_smem + C2 * (C2 + 1));
    float* rdiag = p128_smem + 2 * C2 * (C2 + 1) + 32 * 33;   // 1 / L_ii (after a 32 x 33 scratch)
    const int Mp = cpad128(gs->M);
    const int o = k * C2;
    if (o >= Mp) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    {   // all 16 float4 loads of a thread in flight at once
        float4 v[16];
        #pragma unroll
        for (int u = 0; u < 16; u++) {
            const int idx = tid + u * 256, r = idx >> 5, c = (idx & 31) * 4;
            v[u] = *reinterpret_cast<const float4*>(A + (size_t)(o + r) * ld + o + c);
        }
        #pragma unroll
        for (int u = 0; u < 16; u++) {
            const int idx = tid + u * 256, r = idx >> 5, c = (idx & 31) * 4;
            S[r][c] = (c <= r) ? v[u].x : 0.f;
            S[r][c + 1] = (c + 1 <= r) ? v[u].y : 0.f;
            S[r][c + 2] = (c + 2 <= r) ? v[u].z : 0.f;
            S[r][c + 3] = (c + 3 <= r) ? v[u].w : 0.f;
        }
    }
    __syncthreads();
    for (int p = 0; p < 4; p++) {
        const int c0 = p * 32;
        if (warp == 0) {
            float a[32];
            #pragma unroll
            for (int c = 0; c < 32; c++) a[c] = S[c0 + lane][c0 + c];
            warp_chol32<0>(a, lane, which ? &gs->not_spd_R : &gs->not_spd_F, o + c0);
            #pragma unroll
            for (int c = 0; c < 32; c++) S[c0 + lane][c0 + c] = (c <= lane) ? a[c] : 0.f;
        }
        __syncthreads();
        const int t0 = c0 + 32, below = C2 - t0;
        if (tid < 32) rdiag[c0 + tid] = 1.0f / S[c0 + tid][c0 + tid];
        if (below == 0) break;
        __syncthreads();
        if (tid < below) {                       // rows below: x L_pp^T = a
            const int r = t0 + tid;
            float x[32];
            #pragma unroll
            for (int c = 0; c < 32; c++) x[c] = S[r][c0 + c];
            #pragma unroll
            for (int c = 0; c < 32; c++) {
                float a0 = x[c], a1 = 0.f;
                #pragma unroll
                for (int m = 0; m + 1 < c; m += 2) {
                    a0 -= x[m] * S[c0 + c][c0 + m];
                    a1 -= x[m + 1] * S[c0 + c][c0 + m + 1];
                }
                if (c & 1) a0 -= x[c - 1] * S[c0 + c][c0 + c - 1];
                x[c] = (a0 + a1) * rdiag[c0 + c];
            }
            #pragma unroll
            for (int c = 0; c < 32; c++) S[r][c0 + c] = x[c];
        }
        __syncthreads();
        const int nb = below / 4, nblk = nb * (nb + 1) / 2;
        for (int b = tid; b < nblk; b += blockDim.x) {   // trailing lower triangle, 4x4 blocks
            int bi, bj;
            tri_ij(b, bi, bj);
            const int i0 = t0 + 4 * bi, j0 = t0 + 4 * bj;
            float acc[4][4];
            #pragma unroll
            for (int u = 0; u < 4; u++)
                #pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] = 0.f;
            #pragma unroll 8
            for (int m = 0; m < 32; m++) {
                float ra[4], rb[4];
                #pragma unroll
                for (int u = 0; u < 4; u++) { ra[u] = S[i0 + u][c0 + m]; rb[u] = S[j0 + u][c0 + m]; }
                #pragma unroll
                for (int u = 0; u < 4; u++)
                    #pragma unroll
                    for (int v = 0; v < 4; v++) acc[u][v] += ra[u] * rb[v];
            }
            #pragma unroll
            for (int u = 0; u < 4; u++)
                #pragma unroll
                for (int v = 0; v < 4; v++)
                    if (j0 + v <= i0 + u) S[i0 + u][j0 + v] -= acc[u][v];
        }
        __syncthreads();
    }
    __syncthreads();                 // the last panel's 1/L_ii
    #pragma unroll 4
    for (int u = 0; u < 16; u++) {   // the factor (upper part of the block zero)
        const int idx = tid + u * 256, r = idx >> 5, c = (idx & 31) * 4;
        *reinterpret_cast<float4*>(A + (size_t)(o + r) * ld + o + c) =
            make_float4(S[r][c], S[r][c + 1], S[r][c + 2], S[r][c + 3]);
    }
    // ---- V = L^-1: diagonal 32x32 blocks, one warp each, lane j = column j ----
    if (warp < 4) {
        const int b0 = warp * 32, j = lane;
        float x[32];
        #pragma unroll
        for (int i = 0; i < 32; i++) {
            float acc = (i == j) ? 1.f : 0.f;
            #pragma unroll
            for (int m = 0; m < i; m++) acc -= S[b0 + i][b0 + m] * x[m];
            x[i] = (i < j) ? 0.f : acc * rdiag[b0 + i];
        }
        #pragma unroll
        for (int i = 0; i < 32; i++) V[b0 + i][b0 + j] = x[i];
    }
    __syncthreads();
    // ---- off-diagonal blocks by distance d: V_ij = -V_ii (sum_{k=j}^{i-1} L_ik V_kj) ----
    // The blocks of one distance depend only on nearer ones, so all of them
    // are formed together: two barriers per distance instead of two per
    // block, each sum in its old order.  The products sum_k L_ik V_kj go into
    // the upper triangle of V (block (j, i)), which nothing reads as V.
    for (int d = 1; d < 4; d++) {
        const int nbk = 4 - d;
        for (int e = tid; e < nbk * 32 * 32; e += blockDim.x) {
            const int jb = e >> 10, r = (e >> 5) & 31, c = e & 31, ib = jb + d;
            float acc = 0.f;
            for (int kb = jb; kb < ib; kb++)
                #pragma unroll 8
                for (int m = 0; m < 32; m++) acc += S[ib * 32 + r][kb * 32 + m] * V[kb * 32 + m][jb * 32 + c];
            V[jb * 32 + r][ib * 32 + c] = acc;
        }
        __syncthreads();
        for (int e = tid; e < nbk * 32 * 32; e += blockDim.x) {
            const int jb = e >> 10, r = (e >> 5) & 31, c = e & 31, ib = jb + d;
            float acc = 0.f;
            #pragma unroll 8
            for (int m = 0; m <= r; m++) acc += V[ib * 32 + r][ib * 32 + m] * V[jb * 32 + m][ib * 32 + c];
            V[ib * 32 + r][jb * 32 + c] = -acc;
        }
        __syncthreads();
    }
    // Linv (row-major, upper part zero) and its transpose right after it
    #pragma unroll 4
    for (int u = 0; u < 16; u++) {
        const int idx = tid + u * 256, r = idx >> 5, c = (idx & 31) * 4;
        *reinterpret_cast<float4*>(Linv + (size_t)r * C2 + c) =
            make_float4(c <= r ? V[r][c] : 0.f, c + 1 <= r ? V[r][c + 1] : 0.f, c + 2 <= r ? V[r][c + 2] : 0.f,
                        c + 3 <= r ? V[r][c + 3] : 0.f);
        *reinterpret_cast<float4*>(Linv + C2 * C2 + (size_t)r * C2 + c) =
            make_float4(r <= c ? V[c][r] : 0.f, r <= c + 1 ? V[c + 1][r] : 0.f, r <= c + 2 ? V[c + 2][r] : 0.f,
                        r <= c + 3 ? V[c + 3][r] : 0.f);
    }
}

// One K quarter (32 columns from col) of 128 rows from g0, eight float4 per
// thread, into registers ...
__device__ __forceinline__ void load_quarter(const float* __restrict__ src, size_t lds, int g0, int col,
                                             float4 (&vv)[8])
{
    #pragma unroll
    for (int u = 0; u < 8; u++) {
        const int idx = threadIdx.x + u * 128;
        const int row = idx >> 3, q = idx & 7;
        vv[u] = *reinterpret_cast<const float4*>(src + (size_t)(g0 + row) * lds + col + q * 4);
    }
}

// ... then split into TF32 hi + lo and stored in the SW128 layout of one K block.
__device__ __forceinline__ void store_split_quarter(const float4 (&vv)[8], unsigned char* t_hi, unsigned char* t_lo)
{
    #pragma unroll
    for (int u = 0; u < 8; u++) {
        const int idx = threadIdx.x + u * 128;
        const int row = idx >> 3, kcol = (idx & 7) * 4;
        float x[4] = {vv[u].x, vv[u].y, vv[u].z, vv[u].w};
        float h[4], l[4];
        #pragma unroll
        for (int e = 0; e < 4; e++) {
            uint32_t uu;
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(uu) : "f"(x[e]));
            h[e] = __uint_as_float(uu);
            const float lo = x[e] - h[e];
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(uu) : "f"(lo));
            l[e] = __uint_as_float(uu);
        }
        const uint32_t off = sw128_offset(row, kcol);
        *reinterpret_cast<float4*>(t_hi + off) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(t_lo + off) = make_float4(l[0], l[1], l[2], l[3]);
    }
}

// mode 0: A_IJ -= P_I P_J^T (grid: lower-triangle tiles of the first `band`
// block rows below step k); mode 1: P_I <- P_I Linv^T (grid: block rows).
// K runs in four quarters of 32 columns (the same MMAs in the same order as
// one pass over 128), so a CTA needs 65 KB of shared memory and three fit on
// an SM: while one waits on its loads, the others' MMAs run.  Each quarter's
// global loads are issued while the previous quarter's MMAs run.
__global__ void __launch_bounds__(128, 3) k_chol_tile128(float* __restrict__ A, int ld, int k, GridState* gs, int mode,
                                                         const float* __restrict__ Linv, int band,
                                                         __half* __restrict__ P_hi, __half* __restrict__ P_lo,
                                                         int* __restrict__ pexp)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    const int Mp = cpad128(gs->M);
    const int base = (k + 1) * C2;
    if (base >= Mp) return;
    const int nt = (Mp - base) / C2;
    int I, J = 0;
    if (mode == 0) tri_ij(blockIdx.x, I, J);
    else I = blockIdx.x;
    if (I >= nt || I >= band) return;
    const int r0 = base + I * C2, c0 = base + J * C2;
    const int o = k * C2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    auto tile = [&](int op, int part) { return smem + (op * 2 + part) * TC_TILE_BYTES; };

    if (threadIdx.x == 0) {
        mbar_init(&done_bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bool ok = true;
    float4 ra[8], rb[8];
    load_quarter(A, (size_t)ld, r0, o, ra);
    if (mode == 0) load_quarter(A, (size_t)ld, c0, o, rb);
    else load_quarter(Linv, (size_t)C2, 0, 0, rb);
    for (int qt = 0; qt < 4 && ok; qt++) {
        store_split_quarter(ra, tile(0, 0), tile(0, 1));
        store_split_quarter(rb, tile(1, 0), tile(1, 1));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (warp == 1 && lane == 0) {
            const uint32_t tmem = tmem_slot;
            const uint32_t idesc = idesc_tf32_128x128();
            const uint64_t a_hi = sdesc_sw128(smem_u32(tile(0, 0)));
            const uint64_t a_lo = sdesc_sw128(smem_u32(tile(0, 1)));
            const uint64_t b_hi = sdesc_sw128(smem_u32(tile(1, 0)));
            const uint64_t b_lo = sdesc_sw128(smem_u32(tile(1, 1)));
            #pragma unroll
            for (int kk = 0; kk < TC_KB / 8; kk++) {
                const uint64_t off = (uint64_t)((kk * 32) >> 4);
                mma_tf32(tmem, a_hi + off, b_hi + off, idesc, (qt > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(tmem, a_hi + off, b_lo + off, idesc, 1u);
                mma_tf32(tmem, a_lo + off, b_hi + off, idesc, 1u);
            }
            mma_commit(&done_bar);
        }
        // the next quarter's loads fly while the MMAs run
        if (qt + 1 < 4) {
            load_quarter(A, (size_t)ld, r0, o + (qt + 1) * 32, ra);
            if (mode == 0) load_quarter(A, (size_t)ld, c0, o + (qt + 1) * 32, rb);
            else load_quarter(Linv, (size_t)C2, 0, (qt + 1) * 32, rb);
        }
        __syncthreads();
        // the MMAs read shared memory asynchronously: wait before it is reused
        ok = mbar_wait_bounded(&done_bar, (uint32_t)(qt & 1), &abort_flag, false);
        tc_fence_after();
        __syncthreads();
    }
    const uint32_t tmem = tmem_slot;
    const int row = r0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    const bool good = __syncthreads_and(ok && !abort_flag) != 0;
    if (good && mode == 0) {
        #pragma unroll 1
        for (int c = 0; c < TC_TILE; c += 32) {
            float v[32];
            tmem_ld_32cols(trow + (uint32_t)c, v);
            float* dst = A + (size_t)row * ld + c0 + c;
            #pragma unroll
            for (int i = 0; i < 32; i += 4) {
                float4 a = *reinterpret_cast<float4*>(dst + i);
                a.x -= v[i]; a.y -= v[i + 1]; a.z -= v[i + 2]; a.w -= v[i + 3];
                *reinterpret_cast<float4*>(dst + i) = a;
            }
        }
    } else if (good) {
        // the solved block: FP32 into A, and F16 hi + lo of 2^s x each row (s
        // puts the row's largest entry just below 2^14) into rows 128 I.. of
        // the panel buffer, with s in pexp, for k_chol_upd16
        float mx = 0.f;
        #pragma unroll 1
        for (int c = 0; c < TC_TILE; c += 32) {
            float v[32];
            tmem_ld_32cols(trow + (uint32_t)c, v);
            #pragma unroll
            for (int i = 0; i < 32; i++) mx = fmaxf(mx, fabsf(v[i]));
        }
        int e = 0;
        frexpf(mx, &e);                      // mx < 2^e
        // kept within [-60, 60] so that 2^-(s_i + s_j) is a normal float
        const int sc = (mx > 0.f) ? max(-60, min(60, 14 - e)) : 0;
        pexp[I * C2 + warp * 32 + lane] = sc;
        const float scf = __int_as_float((127 + sc) << 23);
        const size_t prow = (size_t)(I * C2 + warp * 32 + lane) * C2;
        #pragma unroll 1
        for (int c = 0; c < TC_TILE; c += 32) {
            float v[32];
            tmem_ld_32cols(trow + (uint32_t)c, v);
            float* dst = A + (size_t)row * ld + o + c;
            #pragma unroll
            for (int i = 0; i < 32; i += 4)
                *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            uint32_t hw[16], lw[16];
            #pragma unroll
            for (int i = 0; i < 16; i++) {
                const float a = v[2 * i] * scf, b = v[2 * i + 1] * scf;
                const __half ah = __float2half_rn(a), bh = __float2half_rn(b);
                const __half al = __float2half_rn(a - __half2float(ah)), bl = __float2half_rn(b - __half2float(bh));
                hw[i] = (uint32_t)__half_as_ushort(ah) | ((uint32_t)__half_as_ushort(bh) << 16);
                lw[i] = (uint32_t)__half_as_ushort(al) | ((uint32_t)__half_as_ushort(bl) << 16);
            }
            uint4* ph = reinterpret_cast<uint4*>(P_hi + prow + c);
            uint4* pl = reinterpret_cast<uint4*>(P_lo + prow + c);
            #pragma unroll
            for (int q = 0; q < 4; q++) {
                ph[q] = make_uint4(hw[4 * q], hw[4 * q + 1], hw[4 * q + 2], hw[4 * q + 3]);
                pl[q] = make_uint4(lw[4 * q], lw[4 * q + 1], lw[4 * q + 2], lw[4 * q + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (!good && threadIdx.x == 0) atomicExch(&gs->status, QLP_ERR_TIMEOUT);
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
    }
}

// The trailing update of step k, A_IJ -= P_I P_J^T over the lower-triangle
// tiles of the first `band` block rows below the step, from the split panel
// that k_chol_tile128 (mode 1) wrote: map_hi / map_lo address its F16 parts
// ([M_cap rows][128], 64 x 128 boxes, 128-byte swizzle), pexp[row] the
// power-of-two scale of each of its rows.
// K = 128 runs in two halves of 64 (12 MMAs each) through one 64 KB buffer,
// so three CTAs share an SM and overlap each other's loads, MMAs and
// epilogues.
__global__ void __launch_bounds__(128, 3) k_chol_upd16(const __grid_constant__ CUtensorMap map_hi,
                                                       const __grid_constant__ CUtensorMap map_lo,
                                                       float* __restrict__ A, int ld, int k, GridState* gs,
                                                       const int* __restrict__ pexp, int band)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t full_bar, done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    const int Mp = cpad128(gs->M);
    const int base = (k + 1) * C2;
    if (base >= Mp) return;
    const int nt = (Mp - base) / C2;
    int I, J;
    tri_ij(blockIdx.x, I, J);
    if (I >= nt || I >= band) return;
    const int r0 = base + I * C2, c0 = base + J * C2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    auto tile = [&](int op, int part) { return smem + (op * 2 + part) * TC_TILE_BYTES; };
    if (threadIdx.x == 0) {
        mbar_init(&full_bar, 1);
        mbar_init(&done_bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    bool ok = true;
    int issued = 0, landed = 0;      // K halves whose loads were issued / seen complete (thread 0)
    float4 cpre[8];                  // the next 32 columns of this thread's row of the target tile
    for (int h = 0; h < 2; h++) {
        if (threadIdx.x == 0 && !abort_flag) {
            mbar_expect_tx(&full_bar, 4 * TC_TILE_BYTES);
            tma_load_2d(&map_hi, &full_bar, tile(0, 0), h * 64, I * C2);
            tma_load_2d(&map_lo, &full_bar, tile(0, 1), h * 64, I * C2);
            tma_load_2d(&map_hi, &full_bar, tile(1, 0), h * 64, J * C2);
            tma_load_2d(&map_lo, &full_bar, tile(1, 1), h * 64, J * C2);
            issued++;
            if (mbar_wait_bounded(&full_bar, (uint32_t)(h & 1), &abort_flag, false)) {
                landed++;
                tc_fence_after();
                const uint32_t idesc = idesc_f16_128x128();
                const uint64_t a_hi = sdesc_sw128(smem_u32(tile(0, 0)));
                const uint64_t a_lo = sdesc_sw128(smem_u32(tile(0, 1)));
                const uint64_t b_hi = sdesc_sw128(smem_u32(tile(1, 0)));
                const uint64_t b_lo = sdesc_sw128(smem_u32(tile(1, 1)));
                #pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t off = (uint64_t)((kk * 32) >> 4);     // 16 F16 = 32 bytes along K
                    mma_f16(tmem, a_hi + off, b_hi + off, idesc, (h > 0 || kk > 0) ? 1u : 0u);
                    mma_f16(tmem, a_hi + off, b_lo + off, idesc, 1u);
                    mma_f16(tmem, a_lo + off, b_hi + off, idesc, 1u);
                }
            }
            mma_commit(&done_bar);
        }
        __syncthreads();
        // (before the last half's MMAs are waited for, each thread's first
        // 32 columns of the target tile are loaded: their latency overlaps the MMAs)
        if (h == 1) {
            const float* src = A + (size_t)(r0 + warp * 32 + lane) * ld + c0;
            #pragma unroll
            for (int i = 0; i < 8; i++) cpre[i] = *reinterpret_cast<const float4*>(src + 4 * i);
        }
        // the MMAs read shared memory asynchronously: wait before the next half's loads reuse it
        if (!mbar_wait_bounded(&done_bar, (uint32_t)(h & 1), &abort_flag, false)) ok = false;
        tc_fence_after();
        __syncthreads();
    }
    const bool good = __syncthreads_and(ok && !abort_flag) != 0;
    if (good) {
        const int row = r0 + warp * 32 + lane;
        const int si = pexp[I * C2 + warp * 32 + lane];
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        #pragma unroll 1
        for (int c = 0; c < TC_TILE; c += 32) {
            float v[32];
            tmem_ld_32cols(trow + (uint32_t)c, v);
            const int sj = pexp[J * C2 + c + lane];      // column c + lane's row scale, shared through the warp
            float* dst = A + (size_t)row * ld + c0 + c;
            float4 cur[8];
            #pragma unroll
            for (int i = 0; i < 8; i++) cur[i] = cpre[i];
            if (c + 32 < TC_TILE) {                       // the next 32 columns' loads in flight meanwhile
                #pragma unroll
                for (int i = 0; i < 8; i++) cpre[i] = *reinterpret_cast<const float4*>(dst + 32 + 4 * i);
            }
            #pragma unroll
            for (int i = 0; i < 32; i += 4) {
                float4 a = cur[i / 4];
                // 2^-(s_i + s_j), exact (|s_i + s_j| <= 120)
                a.x -= v[i] * __int_as_float((127 - si - __shfl_sync(0xffffffffu, sj, i)) << 23);
                a.y -= v[i + 1] * __int_as_float((127 - si - __shfl_sync(0xffffffffu, sj, i + 1)) << 23);
                a.z -= v[i + 2] * __int_as_float((127 - si - __shfl_sync(0xffffffffu, sj, i + 2)) << 23);
                a.w -= v[i + 3] * __int_as_float((127 - si - __shfl_sync(0xffffffffu, sj, i + 3)) << 23);
                *reinterpret_cast<float4*>(dst + i) = a;
            }
        }
    }
    if (threadIdx.x == 0 && issued > landed)       // copies issued but never seen complete: let them land
        mbar_wait_bounded(&full_bar, (uint32_t)(landed & 1), &abort_flag, false);
    tc_fence_before();
    __syncthreads();
    if (!good && threadIdx.x == 0) atomicExch(&gs->status, QLP_ERR_TIMEOUT);
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
    }
}

// ---------------------------------------------------------------------------
// F z = r with the factor of k_potrf128 / k_chol_tile128 and the inverses of
// its 128x128 diagonal blocks (Linv: per block the inverse and its transpose):
//   forward  y_k = Linv_k (r_k - sum_{j<k} L_kj y_j)
//   backward z_k = Linv_k^T (y_k - sum_{j>k} L_jk^T z_j)
// One CTA per block row; CTA k folds in block j as soon as block j's result
// is published (its flag set with release semantics after the values), so
// the long sums spread over many SMs and only the last block of each sum is
// on the critical path.  Every CTA waits only on CTAs with a smaller index,
// which are scheduled before it (the forward-progress assumption of
// single-pass GPU scans), and every wait is bounded by ~1 s of %globaltimer,
// after which the CTA raises QLP_ERR_TIMEOUT and stops.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits until flags[j] is set, then counts how many of the flags
// j .. jend-1 are set in a row; the count (0 on timeout) is broadcast.
__device__ __forceinline__ int wait_ready(const int* flags, int j, int jend, int step, GridState* gs, int* sh)
{
    if (threadIdx.x == 0) {
        int n = 0;
        if (!ld_acquire(flags + j)) {
            const uint64_t t0 = globaltimer();
            while (!ld_acquire(flags + j)) {
                if (*(volatile int*)&gs->status == QLP_ERR_TIMEOUT) break;     // another CTA gave up
                if (globaltimer() - t0 > TC_WAIT_NS) { atomicExch(&gs->status, QLP_ERR_TIMEOUT); break; }
                __nanosleep(64);
            }
        }
        if (ld_acquire(flags + j)) {
            n = 1;
            for (int q = j + step; q != jend && ld_acquire(flags + q); q += step) n++;
        }
        *sh = n;
    }
    __syncthreads();
    const int n = *sh;
    __syncthreads();
    return n;
}

__global__ void __launch_bounds__(256) k_trsv128_fwd(const float* __restrict__ L, int ld,
                                                     const float* __restrict__ Linv, GridState* gs,
                                                     const double* __restrict__ r, float* y, int* flags)
{
    __shared__ float t[C2];
    __shared__ float red[8][C2 / 8];
    __shared__ int sh;
    const int M = gs->M, nb = cpad128(M) / C2;
    const int k = blockIdx.x;
    if (k >= nb) return;
    const int o = k * C2, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // the diagonal block's inverse rows (two threads per row) and, before each
    // wait, this thread's part of the next block of L's strip are loaded
    // first: their latency overlaps the wait for the block they multiply
    const int irow = tid >> 1, ih = tid & 1;
    float4 lv[16];
    {
        const float4* Lr =
            reinterpret_cast<const float4*>(Linv + (size_t)k * 2 * C2 * C2 + (size_t)irow * C2 + ih * 64);
        #pragma unroll
        for (int u = 0; u < 16; u++) lv[u] = Lr[u];
    }
    float part[16];
    #pragma unroll
    for (int i = 0; i < 16; i++) part[i] = 0.f;
    for (int j = 0; j < k;) {
        float4 lp[16];
        #pragma unroll
        for (int i = 0; i < 16; i++)
            lp[i] = *reinterpret_cast<const float4*>(L + (size_t)(o + warp * 16 + i) * ld + j * C2 + 4 * lane);
        const int n = wait_ready(flags, j, k, 1, gs, &sh);
        if (n == 0) return;
        for (int jj = j; jj < j + n; jj++) {
            const float4 yv = __ldcg(reinterpret_cast<const float4*>(y + (size_t)jj * C2) + lane);
            #pragma unroll
            for (int i = 0; i < 16; i++) {
                const float4 lw = (jj == j) ? lp[i]
                    : *reinterpret_cast<const float4*>(L + (size_t)(o + warp * 16 + i) * ld + jj * C2 + 4 * lane);
                part[i] += lw.x * yv.x + lw.y * yv.y + lw.z * yv.z + lw.w * yv.w;
            }
        }
        j += n;
    }
    #pragma unroll
    for (int i = 0; i < 16; i++)
        for (int off = 16; off > 0; off >>= 1) part[i] += __shfl_xor_sync(0xffffffffu, part[i], off);
    if (lane == 0)
        #pragma unroll
        for (int i = 0; i < 16; i++) red[warp][i] = part[i];
    __syncthreads();
    if (tid < C2) t[tid] = ((o + tid < M) ? (float)r[o + tid] : 0.f) - red[tid >> 4][tid & 15];
    __syncthreads();
    {   // y_k = Linv_k t: two threads per row, a half row each
        float acc = 0.f;
        #pragma unroll
        for (int u = 0; u < 16; u++) {
            const int m = ih * 64 + 4 * u;
            acc += lv[u].x * t[m] + lv[u].y * t[m + 1] + lv[u].z * t[m + 2] + lv[u].w * t[m + 3];
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if (ih == 0) y[o + irow] = acc;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(flags + k, 1);
}

__global__ void __launch_bounds__(256) k_trsv128_bwd(const float* __restrict__ L, int ld,
                                                     const float* __restrict__ Linv, GridState* gs,
                                                     const float* __restrict__ y, float* zf,
                                                     double* __restrict__ zout, int* flags)
{
    __shared__ float t[C2];
    __shared__ float red[8][C2];
    __shared__ int sh;
    const int M = gs->M, nb = cpad128(M) / C2;
    const int b = blockIdx.x;
    if (b >= nb) return;
    const int kb = nb - 1 - b, o = kb * C2, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // as in the forward sweep: the inverse's rows and, before each wait, the
    // next block of L's column strip are loaded first
    const int ic = tid >> 1, ih = tid & 1;
    float4 lv[16];
    {
        const float4* Lr =
            reinterpret_cast<const float4*>(Linv + (size_t)kb * 2 * C2 * C2 + C2 * C2 + (size_t)ic * C2 + ih * 64);
        #pragma unroll
        for (int u = 0; u < 16; u++) lv[u] = Lr[u];
    }
    float4 part = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int j = nb - 1; j > kb;) {
        float4 lp[16];
        #pragma unroll
        for (int i = 0; i < 16; i++)
            lp[i] = *reinterpret_cast<const float4*>(L + (size_t)(j * C2 + warp * 16 + i) * ld + o + 4 * lane);
        const int n = wait_ready(flags, j, kb, -1, gs, &sh);
        if (n == 0) return;
        for (int jj = j; jj > j - n; jj--) {
            #pragma unroll
            for (int i = 0; i < 16; i++) {
                const int row = jj * C2 + warp * 16 + i;
                const float zv = __ldcg(zf + row);
                const float4 lw = (jj == j) ? lp[i] : *reinterpret_cast<const float4*>(L + (size_t)row * ld + o + 4 * lane);
                part.x += lw.x * zv; part.y += lw.y * zv; part.z += lw.z * zv; part.w += lw.w * zv;
            }
        }
        j -= n;
    }
    red[warp][4 * lane] = part.x; red[warp][4 * lane + 1] = part.y;
    red[warp][4 * lane + 2] = part.z; red[warp][4 * lane + 3] = part.w;
    __syncthreads();
    if (tid < C2) {
        float acc = 0.f;
        #pragma unroll
        for (int w = 0; w < 8; w++) acc += red[w][tid];
        t[tid] = y[o + tid] - acc;
    }
    __syncthreads();
    {   // z_k = Linv_k^T t from the stored transpose: two threads per row of it
        float acc = 0.f;
        #pragma unroll
        for (int u = 0; u < 16; u++) {
            const int m = ih * 64 + 4 * u;
            acc += lv[u].x * t[m] + lv[u].y * t[m + 1] + lv[u].z * t[m + 2] + lv[u].w * t[m + 3];
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if (ih == 0) { zf[o + ic] = acc; zout[o + ic] = (double)acc; }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(flags + kb, 1);
}

}  // namespace qlpix
