// Split-FP16 tensor-core GEMM engine on tcgen05 for the precision form of
// the correlation: C (M x N, FP32) = A (M x K) * B (K x N) with
// A = Ahi + Alo and B = Bhi + Blo in FP16 and D = Ahi Bhi + Ahi Blo + Alo Bhi
// accumulated in FP32 in tensor memory (about 22 significant bits per
// operand; the Alo Blo term is below FP32 rounding).
//
// One CTA of 256 threads computes an (MT*128) x NT block over the whole K:
//  * A is a constant matrix prepared once in global memory in the exact
//    shared-memory layout of each K chunk (hi tile then lo tile), so a single
//    1-D bulk copy (TMA) per chunk stages it;
//  * B is produced by the caller's functors (data, split on the fly) and
//    written into the K-major core-matrix layout by six producer warps;
//  * one lane issues the MMAs, tcgen05.commit releases each stage;
//  * the accumulator (MT tiles of 128 lanes x NT columns) is read back with
//    tcgen05.ld by the eight warps and handed to the caller's epilogue.
// Every mbarrier wait is bounded; on a timeout the kernel raises *err and
// every role winds down before tensor memory is freed.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "tc_umma.cuh"

namespace xcg {
namespace tc {

constexpr uint32_t kMaxPolls = 1u << 22;

template <int MT, int NT, int KC>
struct GemmGeom {
    static_assert(KC % 16 == 0 && NT % 16 == 0 && NT >= 16 && NT <= 256, "MMA shape");
    static constexpr uint32_t SBO = (uint32_t)KC * 16u;              // bytes between 8-row groups
    static constexpr uint32_t A_TILE = (uint32_t)MT * 128u * KC * 2u; // one of hi / lo
    static constexpr uint32_t B_TILE = (uint32_t)NT * KC * 2u;
    static constexpr uint32_t STAGE = 2u * A_TILE + 2u * B_TILE;
    static constexpr uint32_t TMEM_COLS_USED = (uint32_t)MT * NT;
    static constexpr uint32_t TMEM_COLS = TMEM_COLS_USED <= 32 ? 32 : TMEM_COLS_USED <= 64 ? 64
                                        : TMEM_COLS_USED <= 128 ? 128 : TMEM_COLS_USED <= 256 ? 256 : 512;
    static_assert(TMEM_COLS_USED <= 512, "tensor memory");
    // dynamic shared memory: two stages + barriers and the tensor-memory address
    static constexpr size_t SMEM = 2 * (size_t)STAGE + 64;
};

// Prepared A in global memory, chunk c at byte offset c * 2 * A_TILE: hi tile,
// then lo tile, each in kmajor_off layout with SBO = 16 * KC.
template <int MT, int NT, int KC>
__host__ __device__ inline size_t prepared_bytes(int K) {
    return (size_t)(K / KC) * 2 * GemmGeom<MT, NT, KC>::A_TILE;
}

// ---------------------------------------------------------------------------
// The block engine: NS stages of one KC-wide K chunk each, filled ahead of
// the tensor core through full/empty mbarrier pairs (no CTA-wide barriers in
// the main loop).
//   warp 0, lane 0: issues the MMAs of chunk c once full[c % NS] has
//     completed, then commits them to empty[c % NS];
//   warp 1, lane 0: bulk-copies A chunk c into its stage (transaction count on
//     full[c % NS]) once the stage is empty;
//   warps 2..7: keep B chunks c+1 and c+2 loading into registers while chunk
//     c is split and stored, fence for the async proxy and arrive on
//     full[c % NS] (one arrival per warp).
// With NS = 4 the producers run up to four chunks ahead of the MMAs.  All
// waits are bounded; a timeout raises *err and every role winds down.
template <int MT, int NT, int NS, int KC_ = 16, int NW = 8>
struct WsGeom {
    static constexpr int KC = KC_;
    static constexpr uint32_t SBO = KC * 16u;
    static constexpr uint32_t A_TILE = (uint32_t)MT * 128u * KC * 2u;
    static constexpr uint32_t B_TILE = (uint32_t)NT * KC * 2u;
    static constexpr uint32_t STAGE = 2u * A_TILE + 2u * B_TILE;
    static constexpr uint32_t TMEM_COLS_USED = (uint32_t)MT * NT;
    static constexpr uint32_t TMEM_COLS = TMEM_COLS_USED <= 32 ? 32 : TMEM_COLS_USED <= 64 ? 64
                                        : TMEM_COLS_USED <= 128 ? 128 : TMEM_COLS_USED <= 256 ? 256 : 512;
    static_assert(TMEM_COLS_USED <= 512 && NT % 16 == 0 && NT <= 256, "shape");
    static_assert(NW >= 4 && NW % 4 == 0, "warps: a multiple of four (TMEM lane quarters)");
    static constexpr int PRODUCERS = (NW - 2) * 32;  // warps 2 .. NW-1
    static constexpr size_t SMEM = (size_t)NS * STAGE + (2 * NS + 1) * 8 + 16;
};

template <int MT, int NT, int NS, bool K_FAST, int KC_ = 16, int NW = 8, class Load, class Cvt, class Epi>
__device__ void gemm_block_ws(const uint8_t *__restrict__ a_prep, int K, Load load, Cvt cvt, Epi epi, int *err) {
    using G = WsGeom<MT, NT, NS, KC_, NW>;
    constexpr int KC = G::KC;
    constexpr int PAIRS = NT * (KC / 2);
    constexpr int ITEMS = (PAIRS + G::PRODUCERS - 1) / G::PRODUCERS;
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(tc_smem + (size_t)NS * G::STAGE);
    uint64_t *empty = full + NS;
    uint64_t *done = empty + NS;
    uint32_t *tmem_sh = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *abort_sh = reinterpret_cast<volatile int *>(tmem_sh + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nchunks = K / KC;

    if (warp == 0) {
        tmem_alloc(tmem_sh, G::TMEM_COLS);
        tmem_relinquish();
    }
    if (tid == 32) {
        for (int i = 0; i < NS; i++) { mbar_init(&full[i], G::PRODUCERS / 32 + 1); mbar_init(&empty[i], 1); }
        mbar_init(done, 1);
        *abort_sh = 0;
        mbar_fence_init();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_sh;
    constexpr uint32_t idesc = idesc_f16_f32(128, NT);

    // the control warps stay converged: lane 0 acts, the other lanes wait at
    // the shuffle instead of polling a barrier beside it
    if (warp == 0) {                                      // MMA issuer
        for (int c = 0; c < nchunks; c++) {
            const int s = c % NS;
            int okw = 1;
            if (lane == 0) {
                if (*abort_sh || !mbar_wait(&full[s], (c / NS) & 1, kMaxPolls)) {
                    *abort_sh = 1;
                    okw = 0;
                } else {
                    fence_after_sync();
                    uint8_t *st = tc_smem + (size_t)s * G::STAGE;
                    const uint32_t a0 = smem_addr(st), b0 = smem_addr(st + 2 * G::A_TILE);
                    const uint64_t bh = sdesc(b0, 128, G::SBO), bl = sdesc(b0 + G::B_TILE, 128, G::SBO);
#pragma unroll 1
                    for (int t = 0; t < MT; t++) {
#pragma unroll
                        for (int j = 0; j < KC / 16; j++) {
                            const uint32_t aoff = (uint32_t)t * 16u * G::SBO + (uint32_t)j * 256u;
                            const uint64_t ahi = sdesc(a0 + aoff, 128, G::SBO);
                            const uint64_t alo = sdesc(a0 + G::A_TILE + aoff, 128, G::SBO);
                            const uint64_t bhj = bh + (uint64_t)((j * 256u) >> 4), blj = bl + (uint64_t)((j * 256u) >> 4);
                            const uint32_t d = tmem + (uint32_t)(t * NT);
                            mma_f16(d, ahi, bhj, idesc, (c > 0 || j > 0) ? 1u : 0u);
                            mma_f16(d, ahi, blj, idesc, 1u);
                            mma_f16(d, alo, bhj, idesc, 1u);
                        }
                    }
                    mma_commit(&empty[s]);
                }
            }
            if (!__shfl_sync(0xffffffffu, okw, 0)) break;
        }
        if (lane == 0) mma_commit(done);                  // everything issued so far, done or not
        __syncwarp();
    } else if (warp == 1) {                               // A producer
        for (int c = 0; c < nchunks; c++) {
            const int s = c % NS;
            int okw = 1;
            if (lane == 0) {
                if (c >= NS && (*abort_sh || !mbar_wait(&empty[s], (c / NS - 1) & 1, kMaxPolls))) {
                    *abort_sh = 1;
                    okw = 0;
                } else {
                    uint8_t *st = tc_smem + (size_t)s * G::STAGE;
                    mbar_expect_tx(&full[s], 2 * G::A_TILE);
                    bulk_g2s(st, a_prep + (size_t)c * 2 * G::A_TILE, 2 * G::A_TILE, &full[s]);
                }
            }
            if (!__shfl_sync(0xffffffffu, okw, 0)) break;
        }
    } else {                                              // B producers
        // loads run two chunks ahead of the stores (register ring of depth 2,
        // the loop unrolled by two so the ring index is static)
        const int p = tid - 64;
        using Raw = decltype(load(0, 0));
        Raw ra[ITEMS], rb[ITEMS];
        auto fetch = [&](Raw *r, int c) {
            if (c >= nchunks) return;
#pragma unroll
            for (int it = 0; it < ITEMS; it++) {
                const int i = p + it * G::PRODUCERS;
                const int n = K_FAST ? i / (KC / 2) : i % NT, k2 = K_FAST ? i % (KC / 2) : i / NT;
                if (i < PAIRS) r[it] = load(c * KC + 2 * k2, n);
            }
        };
        // wait for stage s (warp-uniform), store chunk c from r, publish it
        auto put = [&](Raw *r, int c) -> bool {
            const int s = c % NS;
            if (c >= NS) {
                int okw = 1;
                if (lane == 0) okw = (!*abort_sh && mbar_wait(&empty[s], (c / NS - 1) & 1, kMaxPolls)) ? 1 : 0;
                okw = __shfl_sync(0xffffffffu, okw, 0);
                if (!okw) { if (lane == 0) *abort_sh = 1; return false; }
            }
            uint8_t *st = tc_smem + (size_t)s * G::STAGE;
            __half *bhi = reinterpret_cast<__half *>(st + 2 * G::A_TILE);
            __half *blo = reinterpret_cast<__half *>(st + 2 * G::A_TILE + G::B_TILE);
#pragma unroll
            for (int it = 0; it < ITEMS; it++) {
                const int i = p + it * G::PRODUCERS;
                if (i >= PAIRS) continue;
                const int n = K_FAST ? i / (KC / 2) : i % NT, k2 = K_FAST ? i % (KC / 2) : i / NT;
                const float2 v = cvt(r[it], c * KC + 2 * k2, n);
                __half h0, l0, h1, l1;
                split_f16(v.x, h0, l0);
                split_f16(v.y, h1, l1);
                const uint32_t off = kmajor_off(n, 2 * k2, G::SBO) >> 1;
                *reinterpret_cast<__half2 *>(bhi + off) = __halves2half2(h0, h1);
                *reinterpret_cast<__half2 *>(blo + off) = __halves2half2(l0, l1);
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&full[s]);          // one arrival per producer warp
            return true;
        };
        fetch(ra, 0);
        fetch(rb, 1);
        for (int c = 0; c < nchunks; c += 2) {
            if (!put(ra, c)) break;
            fetch(ra, c + 2);
            if (c + 1 >= nchunks) break;
            if (!put(rb, c + 1)) break;
            fetch(rb, c + 3);
        }
    }
    // the accumulator is complete once `done` has fired (one decision for the CTA)
    const int mine = mbar_wait(done, 0, kMaxPolls) ? 1 : 0;
    const bool ok = __syncthreads_and(mine && !*abort_sh) != 0;
    fence_after_sync();
    if (ok) {
#pragma unroll 1
        for (int t = 0; t < MT; t++) {
#pragma unroll 1
            for (int n0 = 16 * (warp >> 2); n0 < NT; n0 += 16 * (NW / 4)) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(t * NT + n0), v);
                epi(t * 128 + 32 * (warp & 3) + lane, n0, v);
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, G::TMEM_COLS);
}

template <int MT, int NT, int NS, int KC_ = 16>
__host__ __device__ inline size_t ws_prepared_bytes(int K) {
    return (size_t)(K / KC_) * 2 * WsGeom<MT, NT, NS, KC_>::A_TILE;
}

}  // namespace tc
}  // namespace xcg
