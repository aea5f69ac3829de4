// tma.cuh -- the compile-time tile kernel with its tile staged in shared
// memory by the Tensor Memory Accelerator.
//
// The plain tile kernel (tile.cuh) loads its tile with per-thread global
// loads in its first Stockham step. Here one thread copies the CTA's tile
// (C columns x L rows of a column pass, or C rows of a row pass) into a
// staging buffer with cp.async.bulk.tensor, completing on an mbarrier; the
// first step reads its inputs from that buffer (consecutive lanes read
// consecutive words), and the remaining steps and the HBM store of the last
// step are the plain kernel's. A CTA loops over tiles blockIdx.x,
// + gridDim.x, ...; with fewer CTAs than tiles it starts the copy of its next
// tile as soon as the first step has emptied the staging buffer, so that the
// copy overlaps the current tile's remaining steps.
//
// Measured on GB300 (both fields, 2^8- and 2^9-point passes) this is slower
// than the plain kernel: 8-10% with one tile per CTA, more with a persistent
// grid, because the staging buffer costs resident CTAs and every thread waits
// for the whole tile. Plans therefore use the plain kernel unless a caller
// asks for this one (stntt_set_tma).
//
// Tensor maps (built on the host per launch, passed as __grid_constant__):
//   column pass: 3D {S columns, L rows (stride S), Q sub-problems (stride M)},
//     box {C, min(L, 256), 1}; the tile lands as [L][C].
//   row pass: 4D {L, n1 (stride n2 L), n2 (stride L), batch (stride n)} --
//     row r of a transform is input row (r mod n1) n2 + r / n1 -- box
//     {min(L, 256), b1, b2, b3} with b1 b2 b3 = C; the tile lands as
//     [L / 256][C][256] (or [C][L] for L <= 256).
// Every copy starts at an x coordinate that is a multiple of 16 bytes (a
// multiple of C columns with C w >= 16 bytes, or 0 / 256 elements of a row),
// and every wait is bounded: a wait that runs out sets *err and the CTA
// returns (the host reads it with stntt_device_status).
#pragma once
#include <cuda.h>

#include "tile.cuh"

namespace stntt {

struct TmaArgs {
    uint64_t ntiles;       // tiles (CTAs of the plain kernel) over the whole batch
    uint32_t stage_elems;  // offset of the exchange buffer, elements (multiple of 32)
    uint32_t box_bytes;    // bytes of one box (a tile is nbox boxes)
    uint32_t nbox;         // boxes per tile (L / 256 for L > 256, else 1)
    uint32_t spin_limit;   // polls of the mbarrier before giving up
    uint32_t skip_issue;   // self-test only: issue no copy, so the first wait runs out
    uint32_t bar_off;      // byte offset of the mbarrier (and the next tile index after it), 8-byte aligned
    int *err;              // set to 1 when a wait runs out
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t"
        ".reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t"
        "}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Poll the barrier's phase `parity` at most `limit` times (with a short sleep
// after the first 256 polls); false when it did not complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        if (mbar_test(bar, parity))
            return true;
        if (i >= 256)
            __nanosleep(200);
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, uint64_t *bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *tm, uint64_t *bar, int x, int y, int z,
                                            int w) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_addr(bar))
        : "memory");
}

// Issue the copies of tile `blk` into the staging buffer (one thread).
template <class F, int LOGL, int MODE>
__device__ __forceinline__ void tma_issue(const TileArgs<F> &a, const TmaArgs &t, const CUtensorMap *tm,
                                          typename F::T *stage, uint64_t *bar, uint64_t blk) {
    // generic-proxy reads of the staging buffer (ordered by the preceding
    // barrier) before the async-proxy writes of the copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, t.box_bytes * t.nbox);
    const uint64_t gi = blk << a.logC;  // first column (row) of the tile over the batch
    if constexpr (MODE == kModeCol) {
        const uint64_t q = gi >> a.logS;  // sub-problem block over the batch
        const int col = (int)(gi & ((1ull << a.logS) - 1));
        for (uint32_t k = 0; k < t.nbox; ++k)
            tma_load_3d(reinterpret_cast<char *>(stage) + (size_t)k * t.box_bytes, tm, bar, col, (int)(k * 256u),
                        (int)q);
    } else {
        const uint32_t logPer = a.logN - LOGL;  // rows per transform
        const uint64_t b = gi >> logPer;
        const uint64_t rem = gi & ((1ull << logPer) - 1);
        const int y = (int)(rem & ((1ull << a.logN1) - 1));
        const int z = (int)((rem >> a.logN1) & ((1ull << a.logN2) - 1));
        // a tile of more than n1 n2 rows starts a transform and spans the
        // next ones (the box's fourth extent)
        const int w = (int)b;
        for (uint32_t k = 0; k < t.nbox; ++k)
            tma_load_4d(reinterpret_cast<char *>(stage) + (size_t)k * t.box_bytes, tm, bar, (int)(k * 256u), y, z, w);
    }
}

// First-step inputs from the staging buffer; the last step stores to HBM
// exactly as the plain kernel does.
template <class F, bool FULL4, int LOGL, int MODE>
struct StagedIO {
    using T = typename F::T;
    Geo<T> g;
    const T *stage;
    uint32_t c, logC;
    __device__ __forceinline__ T load(uint32_t idx) const {
        if constexpr (MODE == kModeCol) {
            return stage[(idx << logC) + c];
        } else if constexpr (LOGL <= 8) {
            return stage[(c << LOGL) + idx];
        } else {
            return stage[((((idx >> 8) << logC) + c) << 8) + (idx & 255u)];
        }
    }
    __device__ __forceinline__ void store(const TileArgs<F> &a, const F &f, uint32_t pos, T v) const {
        store_last<F, FULL4>(a, f, g, pos, v);
    }
};

template <class F, int LOGL, int MODE, bool FULL4>
__global__ void __launch_bounds__(1024) tile_kernel_tma(const TileArgs<F> a, const __grid_constant__ CUtensorMap tm,
                                                        const TmaArgs t) {
    static_assert(LOGL >= 5, "the first step must not also be the last");
    using T = typename F::T;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    T *stage = reinterpret_cast<T *>(smem_raw);
    T *xchg = stage + t.stage_elems;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + t.bar_off);
    constexpr int TAIL = LOGL & 3;
    constexpr int LOGR0 = TAIL > 0 ? TAIL : 4;
    F f;
    f.p = a.p;

    uint64_t &next_blk = bar[1];  // the next tile, as thread 0 claimed it
    uint64_t blk = blockIdx.x;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        if (blk < t.ntiles && !t.skip_issue)
            tma_issue<F, LOGL, MODE>(a, t, &tm, stage, bar, blk);
    }
    __syncthreads();
    uint32_t phase = 0;
    while (blk < t.ntiles) {
        const bool ok = mbar_wait_bounded(bar, phase, t.spin_limit);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0)
                atomicExch(t.err, 1);
            return;
        }
        phase ^= 1u;
        uint32_t c, u;
        const Geo<T> g = tile_geo<F, 16>(a, blk, c, u);
        // Keep u opaque per tile: otherwise the compiler hoists the step
        // twiddles (which depend only on u) out of the loop and spills them.
        asm volatile("mov.b32 %0, %0;" : "+r"(u));
        const StagedIO<F, FULL4, LOGL, MODE> io{g, stage, c, a.logC};
        T x[16];
        T *col_sm = xchg + c * a.cs;
        // step 0: staging buffer -> registers -> exchange buffer (ends with a barrier)
        tile_step_l<F, 16, LOGL, LOGR0, 0, true, false>(a, f, x, col_sm, u, io);
        // the staging buffer is free: start the next tile's copy
        if (threadIdx.x == 0) {
            const uint64_t nb = blk + gridDim.x;
            next_blk = nb;
            if (nb < t.ntiles)
                tma_issue<F, LOGL, MODE>(a, t, &tm, stage, bar, nb);
        }
        tile_steps_l<F, 16, LOGL, 1>(a, f, x, col_sm, u, io);
        __syncthreads();  // the last step's exchange reads precede the next tile's writes
        blk = next_blk;
    }
}

}  // namespace stntt
