// tc_syrk.cuh -- F = X X^T on the 5th-generation tensor cores (tcgen05).
//
// X is L'^T scaled by sqrt(C^-1): M_cap rows (source cells) x K_cap columns
// (image pixels), K contiguous, split into a rounded high part and a rounded
// remainder so that hi*hi + hi*lo + lo*hi carries ~22 bits.  Two operand
// types, one kernel: TF32 (FP32 storage, kind::tf32, K = 8 per MMA, 32 pixels
// per 128-byte stage row) or F16 (kind::f16 at twice the tensor rate, K = 16
// per MMA, 64 pixels per stage row; X scaled by a power of two so that its
// largest entry is near 2^14, undone exactly in the epilogue).  Both have 11
// significant bits per part.  One CTA computes one 128x128 tile of the lower
// triangle of F:
//   warp 0 / lane 0  TMA producer: 128-row boxes of 128 B (128 B swizzle) of
//                    X_hi, X_lo for the tile's row block and column block
//                    into a 3-stage shared-memory ring;
//   warp 1 / lane 0  MMA issuer: 3 products x 4 k-steps of
//                    tcgen05.mma.cta_group::1 (M=128, N=128) per stage into a
//                    128x128 FP32 accumulator in TMEM;
//   all 4 warps      epilogue: tcgen05.ld 32x32b.x32, FP32 stores to F.
// Block sparsity: a stage is processed only if both the row block and the
// column block of X have a nonzero among its pixels (flags per 32 pixels from
// the PSF-to-X build), so the work follows the overlap of the two source-cell
// blocks' footprints in the image instead of the full pixel count.
// Every mbarrier wait is bounded by ~1 s of %globaltimer; on expiry the
// kernel raises QLP_ERR_TIMEOUT in the GridState, stops issuing work, frees
// its TMEM and returns.
#pragma once
#include "tc_common.cuh"

namespace qlpix {

// grid: one CTA per lower-triangle 128x128 tile of the M_cap x M_cap output.
// nzflags[rb * nkb_cap + kb] != 0 when rows [128 rb, 128 rb + 128) of X have a
// nonzero in columns [32 kb, 32 kb + 32).  HALF: F16 operands (64 pixels per
// stage: flags 2 kb and 2 kb + 1); fscale multiplies the result (2^-2s for X
// scaled by 2^s).
template <bool HALF>
__global__ void __launch_bounds__(128, 1) k_syrk_tc(const __grid_constant__ CUtensorMap map_hi,
                                                    const __grid_constant__ CUtensorMap map_lo,
                                                    GridState* gs, const unsigned char* __restrict__ nzflags,
                                                    int nkb_cap, float* __restrict__ F, int ldF, float fscale)
{
    constexpr int KPS = HALF ? 2 * TC_KB : TC_KB;      // pixels per stage (128 bytes of a row)
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
    const int nkb = (N + KPS - 1) / KPS;

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
    // stage kb has work when both blocks have a nonzero among its pixels
    auto live = [&](int kb) -> bool {
        if (HALF) return (fi[2 * kb] | fi[2 * kb + 1]) && (fj[2 * kb] | fj[2 * kb + 1]);
        return fi[kb] && fj[kb];
    };

    if (warp == 0 && lane == 0) {
        // ---- TMA producer ----
        int it = 0;
        for (int kb = 0; kb < nkb; kb++) {
            if (!live(kb)) continue;
            const int s = it % TC_STAGES;
            if (it >= TC_STAGES) {
                if (!mbar_wait_bounded(&empty_bar[s], ((it / TC_STAGES) & 1) ^ 1, &abort_flag)) break;
            }
            unsigned char* st = smem + s * TC_STAGE_BYTES;
            mbar_expect_tx(&full_bar[s], TC_STAGE_BYTES);
            tma_load_2d(&map_hi, &full_bar[s], st, kb * KPS, bi * TC_TILE);
            tma_load_2d(&map_lo, &full_bar[s], st + TC_TILE_BYTES, kb * KPS, bi * TC_TILE);
            tma_load_2d(&map_hi, &full_bar[s], st + 2 * TC_TILE_BYTES, kb * KPS, bj * TC_TILE);
            tma_load_2d(&map_lo, &full_bar[s], st + 3 * TC_TILE_BYTES, kb * KPS, bj * TC_TILE);
            it++;
        }
        n_issued = it;
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        const uint32_t idesc = HALF ? idesc_f16_128x128() : idesc_tf32_128x128();
        int it = 0;
        for (int kb = 0; kb < nkb; kb++) {
            if (!live(kb)) continue;
            const int s = it % TC_STAGES;
            if (!mbar_wait_bounded(&full_bar[s], (it / TC_STAGES) & 1, &abort_flag)) break;
            tc_fence_after();
            unsigned char* st = smem + s * TC_STAGE_BYTES;
            const uint64_t a_hi = sdesc_sw128(smem_u32(st));
            const uint64_t a_lo = sdesc_sw128(smem_u32(st + TC_TILE_BYTES));
            const uint64_t b_hi = sdesc_sw128(smem_u32(st + 2 * TC_TILE_BYTES));
            const uint64_t b_lo = sdesc_sw128(smem_u32(st + 3 * TC_TILE_BYTES));
            #pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                // one MMA takes 32 bytes along K: 8 TF32 or 16 F16 values
                const uint64_t off = (uint64_t)((kk * 32) >> 4);
                if (HALF) {
                    mma_f16(tmem, a_hi + off, b_hi + off, idesc, (it > 0 || kk > 0) ? 1u : 0u);
                    mma_f16(tmem, a_hi + off, b_lo + off, idesc, 1u);
                    mma_f16(tmem, a_lo + off, b_hi + off, idesc, 1u);
                } else {
                    mma_tf32(tmem, a_hi + off, b_hi + off, idesc, (it > 0 || kk > 0) ? 1u : 0u);
                    mma_tf32(tmem, a_hi + off, b_lo + off, idesc, 1u);
                    mma_tf32(tmem, a_lo + off, b_hi + off, idesc, 1u);
                }
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
                *reinterpret_cast<float4*>(out + c + i) =
                    make_float4(v[i] * fscale, v[i + 1] * fscale, v[i + 2] * fscale, v[i + 3] * fscale);
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

}  // namespace qlpix
