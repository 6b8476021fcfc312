// Split-FP16 tensor-core GEMM engine on tcgen05 for the precision form of
// the correlation: C (M x N, FP32) = A (M x K) * B (K x N) with
// A = Ahi + Alo and B = Bhi + Blo in FP16 and D = Ahi Bhi + Ahi Blo + Alo Bhi
// accumulated in FP32 in tensor memory (about 22 significant bits per
// operand; the Alo Blo term is below FP32 rounding).
//
// One CTA of 128 threads computes an (MT*128) x NT block over the whole K:
//  * A is a constant matrix prepared once in global memory in the exact
//    shared-memory layout of each K chunk (hi tile then lo tile), so a single
//    1-D bulk copy (TMA) per chunk stages it;
//  * B is produced by the caller's functor (data, split on the fly) and
//    written by all threads into the K-major core-matrix layout;
//  * two stages: while the tensor core works on chunk c, the threads stage
//    chunk c+1; stage reuse waits on the MMA commit of chunk c-1;
//  * the accumulator (MT tiles of 128 lanes x NT columns) is read back with
//    tcgen05.ld by the four warps and handed to the caller's epilogue.
// Every mbarrier wait is bounded; on a timeout the kernel raises *err, waits
// (bounded) for its own work in flight, frees tensor memory and returns.
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

// Run the block with NTHR threads (128 or 256).  load(k, n) fetches the raw
// data behind B elements (k, n) and (k+1, n) of this block (k even in [0, K),
// n in [0, NT)); cvt(raw, k, n) -> float2 turns it into the two values,
// already scaled into the FP16 range.  Each thread fetches its share of
// chunk c+1 into registers before the MMAs of chunk c are issued, so global
// latency overlaps the tensor work.  K_FAST: consecutive threads take
// consecutive k pairs (B stored with k contiguous), else consecutive n.
// epi(m, n0, v): the 16 accumulator values of row m (m in [0, MT*128)),
// columns n0..n0+15.
template <int MT, int NT, int KC, int NTHR, bool K_FAST, class Load, class Cvt, class Epi>
__device__ void gemm_block(const uint8_t *__restrict__ a_prep, int K, Load load, Cvt cvt, Epi epi, int *err) {
    using G = GemmGeom<MT, NT, KC>;
    static_assert(NTHR == 128 || NTHR == 256, "threads");
    constexpr int PAIRS = NT * (KC / 2);
    constexpr int ITEMS = (PAIRS + NTHR - 1) / NTHR;
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint8_t *stage_base = tc_smem;
    uint64_t *bar_a = reinterpret_cast<uint64_t *>(tc_smem + 2 * (size_t)G::STAGE);   // [2]
    uint64_t *bar_mma = bar_a + 2;                                                    // [2]
    uint32_t *tmem_sh = reinterpret_cast<uint32_t *>(bar_mma + 2);
    int *abort_sh = reinterpret_cast<int *>(tmem_sh + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nchunks = K / KC;

    if (warp == 0) {
        tmem_alloc(tmem_sh, G::TMEM_COLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&bar_a[0], 1); mbar_init(&bar_a[1], 1);
        mbar_init(&bar_mma[0], 1); mbar_init(&bar_mma[1], 1);
        *abort_sh = 0;
        mbar_fence_init();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_sh;
    constexpr uint32_t idesc = idesc_f16_f32(128, NT);

    using Raw = decltype(load(0, 0));
    Raw raw[ITEMS];
    auto item = [&](int it, int &n, int &k2) {
        const int i = tid + it * NTHR;
        n = K_FAST ? i / (KC / 2) : i % NT;
        k2 = K_FAST ? i % (KC / 2) : i / NT;
        return i < PAIRS;
    };
    auto fetch = [&](int c) {
#pragma unroll
        for (int it = 0; it < ITEMS; it++) {
            int n, k2;
            if (item(it, n, k2)) raw[it] = load(c * KC + 2 * k2, n);
        }
    };
    fetch(0);

    int issued = 0;                       // chunks whose MMAs were committed
    int copied = 0;                       // chunks whose A copy was started
    for (int c = 0; c < nchunks; c++) {
        const int s = c & 1;
        uint8_t *st = stage_base + (size_t)s * G::STAGE;
        // stage s was last read by the MMAs of chunk c-2
        if (c >= 2 && !mbar_wait(&bar_mma[s], ((c - 2) >> 1) & 1, kMaxPolls)) *abort_sh = 1;
        __syncthreads();
        if (*abort_sh) break;
        if (tid == 0) {
            mbar_expect_tx(&bar_a[s], 2 * G::A_TILE);
            bulk_g2s(st, a_prep + (size_t)c * 2 * G::A_TILE, 2 * G::A_TILE, &bar_a[s]);
        }
        copied = c + 1;
        // B chunk: element pairs (k, k+1) of column n -> K-major core layout
        // (adjacent halves of one 16-byte core row), hi and lo tiles
        __half *bhi = reinterpret_cast<__half *>(st + 2 * G::A_TILE);
        __half *blo = reinterpret_cast<__half *>(st + 2 * G::A_TILE + G::B_TILE);
#pragma unroll
        for (int it = 0; it < ITEMS; it++) {
            int n, k2;
            if (!item(it, n, k2)) continue;
            const float2 v = cvt(raw[it], c * KC + 2 * k2, n);
            __half h0, l0, h1, l1;
            split_f16(v.x, h0, l0);
            split_f16(v.y, h1, l1);
            const uint32_t off = kmajor_off(n, 2 * k2, G::SBO) >> 1;
            *reinterpret_cast<__half2 *>(bhi + off) = __halves2half2(h0, h1);
            *reinterpret_cast<__half2 *>(blo + off) = __halves2half2(l0, l1);
        }
        if (c + 1 < nchunks) fetch(c + 1);     // in flight while this chunk's MMAs are issued
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(&bar_a[s], (c >> 1) & 1, kMaxPolls)) {
                *abort_sh = 1;
            } else {
                fence_after_sync();
                const uint32_t a0 = smem_addr(st), b0 = smem_addr(st + 2 * G::A_TILE);
#pragma unroll 1
                for (int t = 0; t < MT; t++) {
#pragma unroll 1
                    for (int j = 0; j < KC / 16; j++) {
                        const uint32_t aoff = (uint32_t)t * 16u * G::SBO + (uint32_t)j * 256u;
                        const uint32_t boff = (uint32_t)j * 256u;
                        const uint64_t ahi = sdesc(a0 + aoff, 128, G::SBO);
                        const uint64_t alo = sdesc(a0 + G::A_TILE + aoff, 128, G::SBO);
                        const uint64_t bh = sdesc(b0 + boff, 128, G::SBO);
                        const uint64_t bl = sdesc(b0 + G::B_TILE + boff, 128, G::SBO);
                        const uint32_t d = tmem + (uint32_t)(t * NT);
                        const uint32_t acc0 = (c > 0 || j > 0) ? 1u : 0u;
                        mma_f16(d, ahi, bh, idesc, acc0);
                        mma_f16(d, ahi, bl, idesc, 1u);
                        mma_f16(d, alo, bh, idesc, 1u);
                    }
                }
                mma_commit(&bar_mma[s]);
            }
        }
        __syncthreads();
        if (*abort_sh) break;
        issued = c + 1;
    }
    // all committed MMAs done (bounded), then the accumulator is read back
    bool ok = !*abort_sh;
    if (issued > 0 && !mbar_wait(&bar_mma[(issued - 1) & 1], ((issued - 1) >> 1) & 1, kMaxPolls)) ok = false;
    if (issued > 1 && !mbar_wait(&bar_mma[(issued - 2) & 1], ((issued - 2) >> 1) & 1, kMaxPolls)) ok = false;
    // an A copy started for a chunk whose MMAs never ran: let it land first
    if (copied > issued && tid == 0) (void)mbar_wait(&bar_a[(copied - 1) & 1], ((copied - 1) >> 1) & 1, kMaxPolls);
    fence_after_sync();
    if (ok && issued == nchunks) {
        // warp w reads lanes 32*(w%4); with 8 warps the two halves take
        // alternate 16-column groups
        constexpr int WG = NTHR / 128;
#pragma unroll 1
        for (int t = 0; t < MT; t++) {
#pragma unroll 1
            for (int n0 = 16 * (warp >> 2); n0 < NT; n0 += 16 * WG) {
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

}  // namespace tc
}  // namespace xcg
