// tc_syrk.cuh -- F = X X^T on the 5th-generation tensor cores (tcgen05, TF32).
//
// X is L'^T scaled by sqrt(C^-1): M_cap rows (source cells) x K_cap columns
// (image pixels), FP32, K contiguous, split into a TF32-rounded high part and
// a TF32-rounded remainder so that hi*hi + hi*lo + lo*hi carries ~22 bits
// (the "3xTF32" scheme).  One CTA computes one 128x128 tile of the lower
// triangle of F:
//   warp 0 / lane 0  TMA producer: 128x32 FP32 boxes (128 B rows, 128 B
//                    swizzle) of X_hi, X_lo for the tile's row block and
//                    column block into a 3-stage shared-memory ring;
//   warp 1 / lane 0  MMA issuer: 3 products x 4 k-steps of
//                    tcgen05.mma.cta_group::1.kind::tf32 (M=128, N=128, K=8)
//                    per stage into a 128x128 FP32 accumulator in TMEM;
//   all 4 warps      epilogue: tcgen05.ld 32x32b.x32, FP32 stores to F.
// Block sparsity: a K block (32 pixels) is processed only if both the row
// block and the column block of X have a nonzero there (flags from the
// conversion kernel), so the work follows the overlap of the two source-cell
// blocks' footprints in the image instead of the full pixel count.
// Every mbarrier wait is bounded by ~1 s of %globaltimer; on expiry the
// kernel raises QLP_ERR_TIMEOUT in the GridState, stops issuing work, frees
// its TMEM and returns.
#pragma once
#include <cuda.h>
#include "qlpix_internal.h"

namespace qlpix {

#define TC_TILE 128
#define TC_KB 32                  // FP32 elements per K block (128 bytes)
#define TC_STAGES 3
#define TC_TILE_BYTES (TC_TILE * TC_KB * 4)          // 16 KB
#define TC_STAGE_BYTES (4 * TC_TILE_BYTES)           // A_hi, A_lo, B_hi, B_lo
#define TC_SMEM (TC_STAGES * TC_STAGE_BYTES + 1024)  // + alignment slack
#define TC_WAIT_NS 1000000000ull

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase: false if ~1 s of %globaltimer ran out
// (the abort flag is then raised) or, when honor_abort is set, as soon as
// another thread of the CTA has given up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, volatile int* abort_flag,
                                                  bool honor_abort = true)
{
    if (mbar_try_wait(bar, phase)) return true;
    const uint64_t t0 = globaltimer();
    while (true) {
        if (mbar_try_wait(bar, phase)) return true;
        if (honor_abort && *abort_flag) return false;
        if (globaltimer() - t0 > TC_WAIT_NS) {
            *abort_flag = 1;
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map, uint64_t* bar, void* dst, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset
    d |= (uint64_t)1 << 46;                 // version
    d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
    return d;
}

// Instruction descriptor: kind::tf32, D=F32, A=B=TF32, both K-major, M=128, N=128.
__device__ __forceinline__ uint32_t idesc_tf32_128x128()
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld_32cols(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    #pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// grid: one CTA per lower-triangle 128x128 tile of the M_cap x M_cap output.
// nzflags[rb * nkb_cap + kb] != 0 when rows [128 rb, 128 rb + 128) of X have a
// nonzero in columns [32 kb, 32 kb + 32).
__global__ void __launch_bounds__(128, 1) k_syrk_tc(const __grid_constant__ CUtensorMap map_hi,
                                                    const __grid_constant__ CUtensorMap map_lo,
                                                    GridState* gs, const unsigned char* __restrict__ nzflags,
                                                    int nkb_cap, float* __restrict__ F, int ldF)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t full_bar[TC_STAGES];
    __shared__ uint64_t empty_bar[TC_STAGES];
    __shared__ uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int n_active;
    __shared__ int n_issued;
    __shared__ volatile int abort_flag;

    int bi, bj;
    {
        int t = blockIdx.x;
        int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
        while ((i + 1) * (i + 2) / 2 <= t) i++;
        while (i * (i + 1) / 2 > t) i--;
        bi = i;
        bj = t - i * (i + 1) / 2;
    }
    const int M = gs->M, N = gs->N;
    const int Mp = (M + TC_TILE - 1) / TC_TILE * TC_TILE;
    if (bi * TC_TILE >= Mp) return;
    const int nkb = (N + TC_KB - 1) / TC_KB;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&done_bar, 1);
        n_active = 0;
        n_issued = 0;
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
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    const unsigned char* fi = nzflags + (size_t)bi * nkb_cap;
    const unsigned char* fj = nzflags + (size_t)bj * nkb_cap;

    if (warp == 0 && lane == 0) {
        // ---- TMA producer ----
        int it = 0;
        for (int kb = 0; kb < nkb; kb++) {
            if (!(fi[kb] && fj[kb])) continue;
            const int s = it % TC_STAGES;
            if (it >= TC_STAGES) {
                if (!mbar_wait_bounded(&empty_bar[s], ((it / TC_STAGES) & 1) ^ 1, &abort_flag)) break;
            }
            unsigned char* st = smem + s * TC_STAGE_BYTES;
            mbar_expect_tx(&full_bar[s], TC_STAGE_BYTES);
            tma_load_2d(&map_hi, &full_bar[s], st, kb * TC_KB, bi * TC_TILE);
            tma_load_2d(&map_lo, &full_bar[s], st + TC_TILE_BYTES, kb * TC_KB, bi * TC_TILE);
            tma_load_2d(&map_hi, &full_bar[s], st + 2 * TC_TILE_BYTES, kb * TC_KB, bj * TC_TILE);
            tma_load_2d(&map_lo, &full_bar[s], st + 3 * TC_TILE_BYTES, kb * TC_KB, bj * TC_TILE);
            it++;
        }
        n_issued = it;
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t idesc = idesc_tf32_128x128();
        int it = 0;
        for (int kb = 0; kb < nkb; kb++) {
            if (!(fi[kb] && fj[kb])) continue;
            const int s = it % TC_STAGES;
            if (!mbar_wait_bounded(&full_bar[s], (it / TC_STAGES) & 1, &abort_flag)) break;
            tc_fence_after();
            unsigned char* st = smem + s * TC_STAGE_BYTES;
            const uint64_t a_hi = sdesc_sw128(smem_u32(st));
            const uint64_t a_lo = sdesc_sw128(smem_u32(st + TC_TILE_BYTES));
            const uint64_t b_hi = sdesc_sw128(smem_u32(st + 2 * TC_TILE_BYTES));
            const uint64_t b_lo = sdesc_sw128(smem_u32(st + 3 * TC_TILE_BYTES));
            #pragma unroll
            for (int kk = 0; kk < TC_KB / 8; kk++) {
                const uint64_t off = (uint64_t)((kk * 32) >> 4);   // 8 TF32 = 32 bytes along K
                mma_tf32(tmem, a_hi + off, b_hi + off, idesc, (it > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(tmem, a_hi + off, b_lo + off, idesc, 1u);
                mma_tf32(tmem, a_lo + off, b_hi + off, idesc, 1u);
            }
            mma_commit(&empty_bar[s]);
            it++;
        }
        n_active = it;
        mma_commit(&done_bar);
    }
    __syncthreads();
    // ---- epilogue ----
    // Wait for the committed MMAs even after an abort: TMEM is freed below.
    const bool ok = mbar_wait_bounded(&done_bar, 0, &abort_flag, false);
    if (abort_flag && threadIdx.x == 0) {
        // let TMA copies that were issued but never consumed land before exit
        for (int it = n_active; it < n_issued; it++)
            mbar_wait_bounded(&full_bar[it % TC_STAGES], (it / TC_STAGES) & 1, &abort_flag, false);
    }
    tc_fence_after();
    const int row = bi * TC_TILE + warp * 32 + lane;
    float* out = F + (size_t)row * ldF + bj * TC_TILE;
    if (ok && !abort_flag && n_active > 0) {
        #pragma unroll 1
        for (int c = 0; c < TC_TILE; c += 32) {
            float v[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
            tmem_ld_32cols(taddr, v);
            #pragma unroll
            for (int i = 0; i < 32; i += 4)
                *reinterpret_cast<float4*>(out + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
    } else {
        for (int c = 0; c < TC_TILE; c += 4) *reinterpret_cast<float4*>(out + c) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    tc_fence_before();
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) atomicExch(&gs->status, QLP_ERR_TIMEOUT);
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
    }
}


// ---------------------------------------------------------------------------
// Trailing update of the FP32 blocked Cholesky on the tensor cores:
//   A_IJ -= P_I P_J^T,   P = L[:, 64k : 64k+64] (the panel just solved),
// for the 128x128 tiles (I >= J) of the trailing lower triangle that starts
// at row/column 64(k+1).  Each CTA loads its two 128x64 panel slices with
// ordinary coalesced loads, splits them into TF32 hi + lo straight into the
// 128-byte-swizzled K-major layout the MMA reads, issues the 3xTF32 products
// (2 K blocks x 4 k-steps x 3) into a TMEM accumulator and subtracts it from
// A in the epilogue.  No waits beyond one bounded mbarrier wait.
// ---------------------------------------------------------------------------
#define UPD_SMEM (4 * TC_TILE_BYTES * 2 + 1024)   // (A,B) x (kb0,kb1) x (hi,lo)

__device__ __forceinline__ uint32_t sw128_offset(int row, int k)
{
    // byte offset of element (row, k) of a [rows][32 floats] K-major tile with 128-byte rows
    const int chunk = (k >> 2) ^ (row & 7);
    return (uint32_t)(row * 128 + chunk * 16 + (k & 3) * 4);
}

__global__ void __launch_bounds__(128, 1) k_chol_update_tc(float* __restrict__ A, int ld, int k, GridState* gs)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    const int Mp = (gs->M + 63) & ~63;
    const int base = (k + 1) * 64;
    if (base >= Mp) return;
    const int nt = (Mp - base + TC_TILE - 1) / TC_TILE;
    int I, J;
    {
        int t = blockIdx.x;
        int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
        while ((i + 1) * (i + 2) / 2 <= t) i++;
        while (i * (i + 1) / 2 > t) i--;
        I = i;
        J = t - i * (i + 1) / 2;
    }
    if (I >= nt) return;
    const int r0 = base + I * TC_TILE, c0 = base + J * TC_TILE;
    const int o = k * 64;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // tiles: [op A/B][kb 0/1][hi/lo], each 128 rows x 128 bytes
    auto tile = [&](int op, int kb, int part) { return smem + ((op * 2 + kb) * 2 + part) * TC_TILE_BYTES; };

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
    // load + split the two 128x64 panel slices (rows beyond Mp read as zero);
    // 8 independent loads in flight per thread
    #pragma unroll 1
    for (int base_idx = threadIdx.x; base_idx < 2 * TC_TILE * 16; base_idx += 8 * 128) {
        float4 vv[8];
        #pragma unroll
        for (int u = 0; u < 8; u++) {
            const int idx = base_idx + u * 128;
            const int op = idx / (TC_TILE * 16);
            const int rem = idx - op * TC_TILE * 16;
            const int row = rem >> 4, q = rem & 15;
            const int grow = (op == 0 ? r0 : c0) + row;
            vv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (grow < Mp) vv[u] = *reinterpret_cast<const float4*>(A + (size_t)grow * ld + o + q * 4);
        }
        #pragma unroll
        for (int u = 0; u < 8; u++) {
            const int idx = base_idx + u * 128;
            const int op = idx / (TC_TILE * 16);
            const int rem = idx - op * TC_TILE * 16;
            const int row = rem >> 4, q = rem & 15;
            const int kb = q >> 3, kcol = (q & 7) * 4;
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
            *reinterpret_cast<float4*>(tile(op, kb, 0) + off) = make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4*>(tile(op, kb, 1) + off) = make_float4(l[0], l[1], l[2], l[3]);
        }
    }
    // make the generic-proxy shared-memory writes visible to the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_tf32_128x128();
        #pragma unroll
        for (int kb = 0; kb < 2; kb++) {
            const uint64_t a_hi = sdesc_sw128(smem_u32(tile(0, kb, 0)));
            const uint64_t a_lo = sdesc_sw128(smem_u32(tile(0, kb, 1)));
            const uint64_t b_hi = sdesc_sw128(smem_u32(tile(1, kb, 0)));
            const uint64_t b_lo = sdesc_sw128(smem_u32(tile(1, kb, 1)));
            #pragma unroll
            for (int kk = 0; kk < TC_KB / 8; kk++) {
                const uint64_t off = (uint64_t)((kk * 32) >> 4);
                mma_tf32(tmem, a_hi + off, b_hi + off, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(tmem, a_hi + off, b_lo + off, idesc, 1u);
                mma_tf32(tmem, a_lo + off, b_hi + off, idesc, 1u);
            }
        }
        mma_commit(&done_bar);
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&done_bar, 0, &abort_flag, false);
    tc_fence_after();
    const int row = r0 + warp * 32 + lane;
    if (ok) {
        #pragma unroll 1
        for (int c = 0; c < TC_TILE; c += 32) {
            float v[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
            tmem_ld_32cols(taddr, v);
            if (row < Mp && c0 + c < Mp) {
                float* dst = A + (size_t)row * ld + c0 + c;
                #pragma unroll
                for (int i = 0; i < 32; i += 4) {
                    float4 a = *reinterpret_cast<float4*>(dst + i);
                    a.x -= v[i]; a.y -= v[i + 1]; a.z -= v[i + 2]; a.w -= v[i + 3];
                    *reinterpret_cast<float4*>(dst + i) = a;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (!ok && threadIdx.x == 0) atomicExch(&gs->status, QLP_ERR_TIMEOUT);
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
    }
}

}  // namespace qlpix
