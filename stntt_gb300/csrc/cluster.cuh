// cluster.cuh -- a whole two-pass transform in one launch: a cluster of K
// CTAs (16 where the device schedules them, else 8) holds it in distributed
// shared memory.
//
// For n = n1 * n2 (n1 = 2^LOG1 column length, n2 = 2^LOG2 row length), the
// same two passes as a two-pass plan (same twiddle tables and arithmetic) run
// back to back inside one cluster per transform:
//   phase 1: CTA r of the cluster takes columns [r n2/K, (r+1) n2/K), reads
//     them from HBM, transforms them and writes each result, after the
//     four-step twiddle, into its own exchange buffer (column-major, odd
//     stride, so that neither these writes nor the phase-2 reads conflict);
//   cluster barrier (every exchange buffer complete);
//   phase 2: CTA r takes rows [r n1/K, (r+1) n1/K); element j of row k1 is
//     element k1 of column j, read from the exchange buffer of CTA j / (n2/K)
//     through distributed shared memory; the row transform's output goes to
//     HBM in the digit-reversed order of the row pass;
//   cluster barrier (no CTA leaves while another still reads its buffer).
// One HBM read and one HBM write per element and one launch, against two of
// each for the two-pass plan: the launch and the second pass's latency are
// what bound single transforms of 2^14..2^17 points.
#pragma once
#include <cooperative_groups.h>

#include "tile.cuh"

namespace stntt {

// Phase 1: loads from HBM (column geometry), stores into the exchange buffer.
template <class F, bool FULL4>
struct ExchangeStoreIO {
    using T = typename F::T;
    Geo<T> g;
    T *xcol;  // this thread's column in the exchange buffer
    __device__ __forceinline__ T load(uint32_t idx) const { return g.valid ? g.src[(uint64_t)idx * g.istride] : T(0); }
    __device__ __forceinline__ void store(const TileArgs<F> &a, const F &f, uint32_t pos, T v) const {
        xcol[pos] = f.canon(four_step<F, FULL4>(a, f, g, pos, v));
    }
};

// Phase 2: loads row `row` from the cluster's exchange buffers, stores to HBM.
template <class F>
struct ClusterGatherIO {
    using T = typename F::T;
    Geo<T> g;
    T *xbuf;  // this CTA's exchange buffer (the same offset in every CTA)
    uint32_t row, logC1, xs;
    __device__ __forceinline__ T load(uint32_t j) const {
        const T *rem = cooperative_groups::this_cluster().map_shared_rank(xbuf, j >> logC1);
        return rem[(j & ((1u << logC1) - 1)) * xs + row];
    }
    __device__ __forceinline__ void store(const TileArgs<F> &a, const F &f, uint32_t pos, T v) const {
        store_last<F, false>(a, f, g, pos, v);
    }
};

// a1 / a2: the plan's two passes, reshaped to n2/K columns and n1/K rows per
// CTA. xoff: element offset of the exchange buffer in shared memory; xs: its
// column stride. Grid: K CTAs per transform, cluster dimension K. E: elements
// per thread of both passes (16, or 8 for twice the threads per CTA).
template <class F, int LOG1, int LOG2, bool FULL4, int E = 16>
__global__ void __launch_bounds__(1024) cluster_kernel(const TileArgs<F> a1, const TileArgs<F> a2, uint32_t xoff,
                                                       uint32_t xs) {
    using T = typename F::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    T *work = reinterpret_cast<T *>(smem_raw);
    T *xbuf = work + xoff;
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    const uint64_t blk = blockIdx.x;  // tile index over the batch: transform blk / K, cluster rank blk mod K
    F f;
    f.p = a1.p;
    T x[E];
    {
        uint32_t c, u;
        const Geo<T> g = tile_geo<F, E>(a1, blk, c, u);
        tile_steps_l<F, E, LOG1, 0, ExchangeStoreIO<F, FULL4>>(a1, f, x, work + c * a1.cs, u,
                                                               ExchangeStoreIO<F, FULL4>{g, xbuf + c * xs});
    }
    cl.sync();
    {
        uint32_t c, u;
        const Geo<T> g = tile_geo<F, E>(a2, blk, c, u);
        const uint32_t row = (uint32_t)(cl.block_rank() << a2.logC) + c;
        tile_steps_l<F, E, LOG2, 0, ClusterGatherIO<F>>(a2, f, x, work + c * a2.cs, u,
                                                        ClusterGatherIO<F>{g, xbuf, row, a1.logC, xs});
    }
    cl.sync();
}

}  // namespace stntt
