// batch.cuh -- one persistent launch for many transforms of uneven sizes.
//
// The host turns a job list into CTA-sized work items (tiles of C columns or
// rows of length L with C * L = 8192, so every item uses 512 threads):
// single-pass jobs of one (size, direction) are packed C transforms per item,
// two-pass jobs contribute their first-pass items and, later in the list,
// their second-pass items. Blocks take items in list order from one atomic
// counter. A second-pass item waits until its job's first-pass items have
// signalled; those were claimed earlier by running blocks that wait on
// nothing, so the wait always ends. Every wait is bounded: past `spin_limit`
// polls the item is skipped, an error flag is set and the host reports
// STNTT_ETIMEOUT.
//
// This extends the reference's uniform `batches` packing
// (src/cuda/ntt/ntt_kernel.cuh:31-39: one n per launch, transforms laid along
// blockDim.y) to mixed sizes, fields' parameters and directions.
#pragma once
#include <cstring>
#include <type_traits>

#include "tile_v.cuh"

namespace stntt {

struct BatchItem {
    uint32_t args;        // index of this item's TileArgs
    uint32_t wait_job;    // job whose first pass must finish first, or ~0u
    uint32_t wait_count;  // number of first-pass items of that job
    uint32_t signal_job;  // job to signal when this item is done, or ~0u
    uint64_t blk;         // CTA index within the item's pass
};

struct BatchCtl {
    unsigned long long next;  // next item to take
    unsigned int error;       // set when a bounded wait gave up
    unsigned int timeouts;
};

constexpr int kBatchThreads = 512;  // C * L / 16 for every item

// One work item with the tile length compiled in, as a called function: its
// registers are allocated on their own, not together with the other lengths'
// bodies and the persistent loop around them.
template <class F, int LOGL>
__device__ __noinline__ void batch_item_l(const TileArgs<F> &a, uint64_t blk, typename F::T *sm) {
    if constexpr (LOGL >= 6) {
        if (a.tw4_full && a.mode == kModeCol) {  // column pass with a full four-step table
            tile_run_l<F, LOGL, true>(a, blk, sm);
            return;
        }
    }
    tile_run_l<F, LOGL>(a, blk, sm);
}

// Tiles of other lengths (2^1..2^3 points: single-pass jobs of up to 8 points).
template <class F>
__device__ __noinline__ void batch_item_small(const TileArgs<F> &sa, uint64_t blk, typename F::T *sm) {
    switch (sa.logL & 3) {
    case 0: tile_run<F, 16, 0>(sa, blk, sm); break;
    case 1: tile_run<F, 16, 1>(sa, blk, sm); break;
    case 2: tile_run<F, 16, 2>(sa, blk, sm); break;
    default: tile_run<F, 16, 3>(sa, blk, sm); break;
    }
}

// An item of a two-pass job in the vector-lines layout (tile_v.cuh): C =
// 8192 / L lines of one job, V adjacent lines per thread (16 bytes: two
// Goldilocks values with 8 points each, or four 32-bit values with 4 points
// each, so 512 threads either way), 16-byte HBM accesses; a column item
// carries its four-step twiddle in a full table. Geometry as in
// tile_kernel_v, with the job's data reached through the item's pointer
// arrays.
template <class F>
__host__ __device__ constexpr int batch_vlines() {
    return sizeof(typename F::T) == 8 ? 2 : 4;
}
template <class F, int LOGL, bool COL>
__device__ __noinline__ void batch_item_vec(const TileArgs<F> &a, uint64_t blk, typename F::T *sm) {
    using T = typename F::T;
    constexpr int V = batch_vlines<F>(), E = 16 / V, LOGG = 13 - LOGL - (V == 2 ? 1 : 2);
    static_assert(LOGG >= 0 && (1u << LOGG) * ((1u << LOGL) / E) == kBatchThreads, "512 threads per item");
    constexpr uint32_t G = 1u << LOGG, C = V * G;
    const uint32_t g = threadIdx.x & (G - 1), u = threadIdx.x >> LOGG;
    F f;
    f.p = a.p;
    const uint64_t line0 = blk * C + g * V;
    const uint32_t logPer = a.logN - LOGL;
    const uint64_t b = line0 >> logPer, rem = line0 & ((1ull << logPer) - 1);
    const T *ibase = reinterpret_cast<const T *>(a.in_ptrs[b]);
    T *obase = reinterpret_cast<T *>(a.out_ptrs[b]);
    VGeo<T, V> geo;
    if constexpr (COL) {
        const uint64_t q = rem >> a.logS;
        geo.col0 = (uint32_t)(rem & ((1ull << a.logS) - 1));
        geo.src[0] = ibase + (q << a.logM) + geo.col0;
#pragma unroll
        for (int i = 1; i < V; ++i)
            geo.src[i] = geo.src[0];
        geo.dst = obase + (q << a.logM) + geo.col0;
        geo.istride = geo.ostride = 1u << a.logS;
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) {
            const uint64_t r = rem + i;
            const uint64_t inrow = ((r & ((1ull << a.logN1) - 1)) << a.logN2) + (r >> a.logN1);
            geo.src[i] = ibase + (inrow << LOGL);
        }
        geo.dst = obase + rem;
        geo.istride = 1;
        geo.ostride = 1u << logPer;
        geo.col0 = 0;
    }
    T x[V][E];
    vsteps<F, V, E, LOGL, LOGG, 0, COL, COL ? 1 : 0>(a, f, x, sm + g * V, u, geo);
}

template <class F, bool COL>
__device__ __forceinline__ void batch_item_vec_l(const TileArgs<F> &sa, uint64_t blk, typename F::T *sm) {
    switch (sa.logL) {
    case 4: batch_item_vec<F, 4, COL>(sa, blk, sm); break;
    case 5: batch_item_vec<F, 5, COL>(sa, blk, sm); break;
    case 6: batch_item_vec<F, 6, COL>(sa, blk, sm); break;
    case 7: batch_item_vec<F, 7, COL>(sa, blk, sm); break;
    case 8: batch_item_vec<F, 8, COL>(sa, blk, sm); break;
    case 9: batch_item_vec<F, 9, COL>(sa, blk, sm); break;
    case 10: batch_item_vec<F, 10, COL>(sa, blk, sm); break;
    case 11: batch_item_vec<F, 11, COL>(sa, blk, sm); break;
    default: break;  // the host sets vecl only for 2^4..2^11-point passes
    }
}

template <class F>
__host__ __device__ constexpr bool batch_vec_field() {
    return IsPow2Field<F>::value || std::is_same_v<F, FieldU32L>;
}

// One item of any tile length (every item: 16 elements per thread, or the
// vector-lines layout where the host marked the pass).
template <class F>
__device__ __forceinline__ void batch_item(const TileArgs<F> &sa, uint64_t blk, typename F::T *sm) {
    if constexpr (batch_vec_field<F>()) {
        if (sa.vecl == (uint32_t)batch_vlines<F>()) {
            if (sa.mode == kModeCol)
                batch_item_vec_l<F, true>(sa, blk, sm);
            else
                batch_item_vec_l<F, false>(sa, blk, sm);
            return;
        }
    }
    switch (sa.logL) {
    case 4: batch_item_l<F, 4>(sa, blk, sm); break;
    case 5: batch_item_l<F, 5>(sa, blk, sm); break;
    case 6: batch_item_l<F, 6>(sa, blk, sm); break;
    case 7: batch_item_l<F, 7>(sa, blk, sm); break;
    case 8: batch_item_l<F, 8>(sa, blk, sm); break;
    case 9: batch_item_l<F, 9>(sa, blk, sm); break;
    case 10: batch_item_l<F, 10>(sa, blk, sm); break;
    case 11: batch_item_l<F, 11>(sa, blk, sm); break;
    case 12: batch_item_l<F, 12>(sa, blk, sm); break;
    case 13: batch_item_l<F, 13>(sa, blk, sm); break;
    default: batch_item_small<F>(sa, blk, sm); break;
    }
}

// The current item's descriptor in shared memory. Goldilocks launches mix
// directions, so their items get the descriptor as the direction-specialised
// field type (FieldGLF / FieldGLI: shift-only internal twiddles; same
// layout), chosen per item by TileArgs::pow2 (the host admits only the two
// standard roots).
template <class F>
struct BatchArgsSm {
    TileArgs<F> a;
};
template <>
struct BatchArgsSm<FieldGL> {
    TileArgs<FieldGL> a;
    TileArgs<FieldGLF> f;
    TileArgs<FieldGLI> i;
};

template <class F, int MINB = 2>
__global__ void __launch_bounds__(kBatchThreads, MINB) batch_kernel(const TileArgs<F> *__restrict__ args,
                                                              const BatchItem *__restrict__ items,
                                                              unsigned long long nitems, unsigned int *counters,
                                                              BatchCtl *ctl, unsigned int spin_limit) {
    using T = typename F::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ BatchArgsSm<F> sargs;
    TileArgs<F> &sa = sargs.a;
    __shared__ unsigned long long s_item;
    __shared__ int s_ok;
    T *sm = reinterpret_cast<T *>(smem_raw);
    for (;;) {
        if (threadIdx.x == 0)
            s_item = atomicAdd(&ctl->next, 1ull);
        __syncthreads();
        const unsigned long long it = s_item;
        if (it >= nitems)
            break;
        const BatchItem bi = items[it];
        if (threadIdx.x == 0) {
            int ok = 1;
            if (bi.wait_job != ~0u) {
                unsigned int spins = 0;
                while (atomicAdd(&counters[bi.wait_job], 0u) < bi.wait_count) {
                    if (++spins > spin_limit) {
                        ok = 0;
                        atomicExch(&ctl->error, 1u);
                        atomicAdd(&ctl->timeouts, 1u);
                        break;
                    }
                    __nanosleep(200);
                }
                __threadfence();
            }
            s_ok = ok;
            sa = args[bi.args];
            if constexpr (std::is_same_v<F, FieldGL>) {
                static_assert(sizeof(TileArgs<FieldGLF>) == sizeof(TileArgs<FieldGL>), "same descriptor layout");
                if (sa.pow2 == 2)
                    memcpy(&sargs.i, &sa, sizeof(sa));
                else
                    memcpy(&sargs.f, &sa, sizeof(sa));
            }
        }
        __syncthreads();
        if (s_ok) {
            if constexpr (std::is_same_v<F, FieldGL>) {
                if (sa.pow2 == 2)
                    batch_item<FieldGLI>(sargs.i, bi.blk, sm);
                else
                    batch_item<FieldGLF>(sargs.f, bi.blk, sm);
            } else {
                batch_item<F>(sa, bi.blk, sm);
            }
        }
        __threadfence();  // this item's stores before the signal below
        __syncthreads();
        if (threadIdx.x == 0 && bi.signal_job != ~0u)
            atomicAdd(&counters[bi.signal_job], 1u);
    }
}

}  // namespace stntt
