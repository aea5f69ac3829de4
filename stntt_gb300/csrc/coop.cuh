// coop.cuh -- both passes of a two-pass plan in one cooperative launch, for
// single transforms of 2^16..2^21 points whose passes are one wave of CTAs.
//
// Each CTA runs its first-pass tiles (column pass, four-step twiddle on the
// way out), waits at a grid-wide barrier, then runs its second-pass tiles
// (row pass, digit-reversed output). The cooperative launch guarantees that
// every CTA is resident, so the barrier cannot deadlock; its spin is bounded
// all the same (about a second of polls), after which the CTA records an
// error in the context's device word and goes on (the output is then
// incomplete; stntt_device_status reports STNTT_ETIMEOUT). One launch instead
// of two removes the second launch's latency and the ramp between the passes,
// the cost of a lone transform of this size (each pass fills the GPU once).
//
// The barrier is a counter and a sense word kept in the tail of the stream's
// workspace (calls on one stream are ordered, so they never share it
// concurrently): each CTA reads the sense, then adds one to the counter; the
// last to arrive clears the counter and flips the sense, which releases the
// others. The counter is zero again when the kernel ends.
//
// Replaces, like tile.cuh, the reference's one-launch-per-stage global passes
// (sttNttGlobalRadix2, st_ntt_global_radix2.cuh:88-117), which also separate
// their launches with a host synchronisation (:108, :111).
#pragma once
#include <cstdint>

#include "tile.cuh"

namespace stntt {

struct CoopBarrier {
    unsigned int count;
    unsigned int sense;
};

// Grid-wide barrier (see above); every thread of the CTA calls it.
__device__ __forceinline__ void coop_grid_sync(CoopBarrier *bar, unsigned int nblocks, int *err,
                                               unsigned int spin_limit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *sense = &bar->sense;
        const unsigned int s = *sense;
        __threadfence();  // this CTA's first-pass stores before its arrival
        const unsigned int c = atomicAdd(&bar->count, 1u);
        if (c + 1 == nblocks) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicExch(&bar->sense, s ^ 1u);
        } else {
            unsigned int spins = 0;
            while (*sense == s) {
                if (++spins > spin_limit) {
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();  // the other CTAs' stores before this CTA's second pass
    }
    __syncthreads();
}

// a1: the column pass (input -> workspace), a2: the row pass (workspace ->
// output); both with threads == C * L / E.
template <class F, int LOG1, int LOG2, int E>
__global__ void __launch_bounds__(512) coop_kernel(const TileArgs<F> a1, const TileArgs<F> a2, CoopBarrier *bar,
                                                   int *err, unsigned int spin_limit) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using T = typename F::T;
    T *sm = reinterpret_cast<T *>(smem_raw);
    const uint64_t tiles1 = a1.total >> a1.logC, tiles2 = a2.total >> a2.logC;
    for (uint64_t t = blockIdx.x; t < tiles1; t += gridDim.x) {
        tile_run_l<F, LOG1, false, E>(a1, t, sm);
        __syncthreads();
    }
    coop_grid_sync(bar, gridDim.x, err, spin_limit);
    for (uint64_t t = blockIdx.x; t < tiles2; t += gridDim.x) {
        tile_run_l<F, LOG2, false, E>(a2, t, sm);
        __syncthreads();
    }
}

}  // namespace stntt
