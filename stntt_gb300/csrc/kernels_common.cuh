// kernels_common.cuh -- field-generic kernels and launchers, instantiated once
// per field by kernels_u32.cu and kernels_gl64.cu.
#pragma once
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <utility>

#include "batch.cuh"
#include "cluster.cuh"
#include "internal.h"
#include "tile.cuh"

namespace stntt {

template <class F>
__device__ __forceinline__ typename F::TW to_tw(uint64_t raw) {
    typename F::TW w;
    memcpy(&w, &raw, sizeof(w));
    return w;
}

// Raise one tile kernel's dynamic shared-memory limit, once per device. The
// call also loads the kernel's code, so the first launch does not.
template <class F, auto KERN>
cudaError_t tile_attr() {
    static bool attr_set[64] = {};  // per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        e = cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess)
            return e;
        attr_set[dev] = true;
    }
    return cudaSuccess;
}

// Programmatic dependent launch for the passes of calls of at least 2^22
// elements: measured on GB300, Goldilocks 2^24 forward + inverse 729 -> 716 us
// and 32-bit 2^26 1324 -> 1312 us per step, while replayed graphs of 2^20-point
// transforms became slower (85 -> 91 us), so smaller calls launch plainly.
constexpr uint64_t kPdlMinElems = 1ull << 22;
// kPdlMinElems, or 2^STNTT_PDL_MIN_LOG (0..40) from the environment (read once).
inline uint64_t pdl_min_elems() {
    static const uint64_t v = [] {
        const char *e = getenv("STNTT_PDL_MIN_LOG");
        const long x = e ? strtol(e, nullptr, 10) : -1;
        return (x >= 0 && x <= 40) ? (1ull << x) : kPdlMinElems;
    }();
    return v;
}

template <class F, auto KERN>
cudaError_t launch_tile_k(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    cudaError_t e = tile_attr<F, KERN>();
    if (e != cudaSuccess)
        return e;
    if (d.smem_bytes > 200 * 1024)
        return cudaErrorInvalidConfiguration;
    if ((a.total << d.logL) < pdl_min_elems()) {
        KERN<<<(unsigned)blocks, d.threads, d.smem_bytes, s>>>(a);
        return cudaGetLastError();
    }
    // Programmatic dependent launch: this pass's CTAs may be scheduled while
    // the previous kernel finishes; the kernel waits (griddepcontrol.wait)
    // before it reads or writes global memory.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(d.threads);
    cfg.dynamicSmemBytes = d.smem_bytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, KERN, a);
    return e == cudaSuccess ? cudaGetLastError() : e;
}


template <class F, int E, int TAIL, bool IN2 = false>
cudaError_t launch_tile_e(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    return launch_tile_k<F, tile_kernel<F, E, TAIL, IN2>>(d, a, blocks, s);
}

// Tile lengths 2^4..2^13 at 16 elements per thread: the kernel with the
// length compiled in (column passes with a full four-step table from 2^6 up:
// the FULL4 build). false when logL is outside that range.
// 32-bit lazy-field passes of at most 256 threads per CTA run the build with
// six CTAs resident per SM (at most 40 registers, no spills): 32-bit 2^26
// forward + inverse 1354 -> 1269 us per step on GB300 (eight per SM: 1274 us,
// with spills). Goldilocks passes keep 64 registers (five per SM spilled and
// ran 11% slower).
constexpr int kU32MinBlocks = 6;

template <class F, int LOGL, int MINB>
cudaError_t launch_tile_lm(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    if constexpr (LOGL >= 6) {
        if (a.tw4_full && a.mode == kModeCol)
            return launch_tile_k<F, tile_kernel_l<F, LOGL, true, MINB>>(d, a, blocks, s);
    }
    return launch_tile_k<F, tile_kernel_l<F, LOGL, false, MINB>>(d, a, blocks, s);
}

template <class F, int LOGL>
cudaError_t launch_tile_l(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    if constexpr (std::is_same_v<F, FieldU32L>) {
        if (d.threads <= 256)
            return launch_tile_lm<F, LOGL, kU32MinBlocks>(d, a, blocks, s);
    }
    return launch_tile_lm<F, LOGL, 1>(d, a, blocks, s);
}

// Eight elements per thread (twice the threads of a 16-element tile), tile
// lengths 2^7..2^11: passes of small transforms, where the SMs hold too few
// warps at 16 elements per thread.
template <class F, int LOGL>
cudaError_t launch_tile_l8(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    if (a.tw4_full && a.mode == kModeCol)
        return launch_tile_k<F, tile_kernel_l<F, LOGL, true, 1, 8>>(d, a, blocks, s);
    return launch_tile_k<F, tile_kernel_l<F, LOGL, false, 1, 8>>(d, a, blocks, s);
}

template <class F>
bool launch_tile_fixed8(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s, cudaError_t *e) {
    switch (d.logL) {
    case 7: *e = launch_tile_l8<F, 7>(d, a, blocks, s); return true;
    case 8: *e = launch_tile_l8<F, 8>(d, a, blocks, s); return true;
    case 9: *e = launch_tile_l8<F, 9>(d, a, blocks, s); return true;
    case 10: *e = launch_tile_l8<F, 10>(d, a, blocks, s); return true;
    case 11: *e = launch_tile_l8<F, 11>(d, a, blocks, s); return true;
    default: return false;
    }
}

template <class F>
bool launch_tile_fixed(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s, cudaError_t *e) {
    switch (d.logL) {
    case 4: *e = launch_tile_l<F, 4>(d, a, blocks, s); return true;
    case 5: *e = launch_tile_l<F, 5>(d, a, blocks, s); return true;
    case 6: *e = launch_tile_l<F, 6>(d, a, blocks, s); return true;
    case 7: *e = launch_tile_l<F, 7>(d, a, blocks, s); return true;
    case 8: *e = launch_tile_l<F, 8>(d, a, blocks, s); return true;
    case 9: *e = launch_tile_l<F, 9>(d, a, blocks, s); return true;
    case 10: *e = launch_tile_l<F, 10>(d, a, blocks, s); return true;
    case 11: *e = launch_tile_l<F, 11>(d, a, blocks, s); return true;
    case 12: *e = launch_tile_l<F, 12>(d, a, blocks, s); return true;
    case 13: *e = launch_tile_l<F, 13>(d, a, blocks, s); return true;
    default: return false;
    }
}

// ---- one-launch transforms in a thread-block cluster (cluster.cuh)
// Shared-memory limit and permission for 16-CTA clusters, once per device.
template <class F, auto KERN>
cudaError_t cluster_attr() {
    static bool attr_set[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        e = cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(KERN, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess)
            return e;
        attr_set[dev] = true;
    }
    return cudaSuccess;
}

template <class F, int LOG1, int LOG2, int E = 16>
cudaError_t launch_cluster_k(const TileArgs<F> &a1, const TileArgs<F> &a2, uint32_t xoff, uint32_t xs,
                             uint64_t blocks, uint32_t threads, size_t smem, uint32_t log_k, cudaStream_t s) {
    auto kern = cluster_kernel<F, LOG1, LOG2, true, E>;
    cudaError_t e = cluster_attr<F, cluster_kernel<F, LOG1, LOG2, true, E>>();
    if (e != cudaSuccess)
        return e;
    if (smem > 200 * 1024 || blocks > 0x7fffffffull)
        return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1u << log_k;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, a1, a2, xoff, xs);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

template <class F>
void fill_args(TileArgs<F> &a, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out) {
    using T = typename F::T;
    using TW = typename F::TW;
    const TW *tab = static_cast<const TW *>(tables);
    a.in = static_cast<const T *>(in);
    a.out = static_cast<T *>(out);
    a.twL = tab + d.tw_off;
    a.tw4_lo = tab + d.lo_off;
    a.tw4_hi = tab + d.hi_off;
    a.tw4_full = (d.full_off == ~0ull || d.full_mont) ? nullptr : tab + d.full_off;
    a.tw4_mont = (d.full_off != ~0ull && d.full_mont) ? reinterpret_cast<const uint32_t *>(tab + d.full_off) : nullptr;
    a.pinv = d.pinv;
    a.pow2 = d.pow2;
    a.vecl = d.vec;
    for (int j = 0; j < 8; ++j)
        std::memcpy(&a.wR[j], &d.wR[j], sizeof(TW));
    std::memcpy(&a.scale, &d.scale, sizeof(TW));
    a.p = p;
    a.logL = d.logL;
    a.logC = d.logC;
    a.mode = d.mode;
    a.do_scale = d.do_scale;
    a.tfast = d.tfast;
    a.h = d.h;
    a.logN = d.logN;
    a.logM = d.logM;
    a.logS = d.logS;
    a.logN1 = d.logN1;
    a.logN2 = d.logN2;
    a.cs = d.cs;
    a.in_ptrs = nullptr;
    a.out_ptrs = nullptr;
    a.in2 = nullptr;
    a.total = 0;
}

// The TMA-staged persistent kernel (tma.cuh) for one pass, defined per field
// in kernels_tma_*.cu; cudaErrorNotSupported when the pass cannot use it
// (then the plain kernel runs).
cudaError_t launch_tma_gl64(const PassDesc &d, const TileArgs<FieldGL> &a, uint64_t batch, uint64_t tiles, int *err,
                            cudaStream_t s);
cudaError_t launch_tma_u32l(const PassDesc &d, const TileArgs<FieldU32L> &a, uint64_t batch, uint64_t tiles,
                            int *err, cudaStream_t s);
template <class F>
cudaError_t launch_tma(const PassDesc &d, const TileArgs<F> &a, uint64_t batch, uint64_t tiles, int *err,
                       cudaStream_t s) {
    if constexpr (std::is_same_v<F, FieldGL>) {
        return launch_tma_gl64(d, a, batch, tiles, err, s);
    } else if constexpr (IsPow2Field<F>::value) {
        // the staged kernel keeps product internal twiddles (same descriptor)
        static_assert(sizeof(TileArgs<F>) == sizeof(TileArgs<FieldGL>), "same descriptor layout");
        TileArgs<FieldGL> g;
        std::memcpy(&g, &a, sizeof(g));
        return launch_tma_gl64(d, g, batch, tiles, err, s);
    } else if constexpr (std::is_same_v<F, FieldU32L>)
        return launch_tma_u32l(d, a, batch, tiles, err, s);
    else
        return cudaErrorNotSupported;
}

template <class F>
cudaError_t launch_tile_t(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                          uint64_t batch, cudaStream_t s, const void *in2 = nullptr, int *err = nullptr) {
    TileArgs<F> a;
    fill_args<F>(a, d, p, tables, in, out);
    a.in2 = static_cast<const typename F::T *>(in2);
    const uint64_t rows = batch << (d.logN - d.logL);
    a.total = rows;
    const uint64_t blocks = (rows + (1ull << d.logC) - 1) >> d.logC;
    if (blocks == 0)
        return cudaSuccess;
    if (blocks > 0x7fffffffull)
        return cudaErrorInvalidConfiguration;
    if (d.tma && err && !in2) {
        const cudaError_t e = launch_tma<F>(d, a, batch, blocks, err, s);
        if (e != cudaErrorNotSupported)
            return e;
    }
    const uint32_t tail = d.logL & 3;
    if (in2) {  // fused pointwise product: instantiated for up to 16 elements per thread
        switch (d.E) {
        case 2: return launch_tile_e<F, 2, 1, true>(d, a, blocks, s);
        case 4: return launch_tile_e<F, 4, 2, true>(d, a, blocks, s);
        case 8: return launch_tile_e<F, 8, 3, true>(d, a, blocks, s);
        case 16:
            switch (tail) {
            case 0: return launch_tile_e<F, 16, 0, true>(d, a, blocks, s);
            case 1: return launch_tile_e<F, 16, 1, true>(d, a, blocks, s);
            case 2: return launch_tile_e<F, 16, 2, true>(d, a, blocks, s);
            default: return launch_tile_e<F, 16, 3, true>(d, a, blocks, s);
            }
        default: return cudaErrorNotSupported;
        }
    }
    cudaError_t e;
    if (d.E == 16 && launch_tile_fixed<F>(d, a, blocks, s, &e))
        return e;
    if (d.E == 8 && (1u << d.logL) > 8) {  // the generic build's 8-element tiles hold one step only
        if (launch_tile_fixed8<F>(d, a, blocks, s, &e))
            return e;
        return cudaErrorNotSupported;
    }
    switch (d.E) {
    case 2: return launch_tile_e<F, 2, 1>(d, a, blocks, s);
    case 4: return launch_tile_e<F, 4, 2>(d, a, blocks, s);
    case 8: return launch_tile_e<F, 8, 3>(d, a, blocks, s);
    case 16:
        switch (tail) {
        case 0: return launch_tile_e<F, 16, 0>(d, a, blocks, s);
        case 1: return launch_tile_e<F, 16, 1>(d, a, blocks, s);
        case 2: return launch_tile_e<F, 16, 2>(d, a, blocks, s);
        default: return launch_tile_e<F, 16, 3>(d, a, blocks, s);
        }
    case 32:
        switch (tail) {
        case 0: return launch_tile_e<F, 32, 0>(d, a, blocks, s);
        case 1: return launch_tile_e<F, 32, 1>(d, a, blocks, s);
        case 2: return launch_tile_e<F, 32, 2>(d, a, blocks, s);
        default: return launch_tile_e<F, 32, 3>(d, a, blocks, s);
        }
    default: return cudaErrorInvalidValue;
    }
}

// Both passes of a two-pass plan in one launch of clusters of 2^log_k CTAs:
// d1 / d2 already hold n2 / K columns and n1 / K rows per CTA. cudaErrorNotSupported when this split
// (tile lengths 2^7..2^9, n = 2^14..2^17) or a missing full four-step table
// rules it out; the caller then launches the two passes.
template <class F>
cudaError_t launch_cluster_t(const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables, const void *in,
                             void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem, uint32_t log_k,
                             cudaStream_t s) {
    TileArgs<F> a1, a2;
    fill_args<F>(a1, d1, p, tables, in, nullptr);
    fill_args<F>(a2, d2, p, tables, nullptr, out);
    a1.total = batch << (d1.logN - d1.logL);
    a2.total = batch << (d2.logN - d2.logL);
    if (!a1.tw4_full)
        return cudaErrorNotSupported;
    const uint64_t blocks = batch << log_k;
    const uint32_t t = d1.threads;
    if (d1.E == 8) {  // 8 elements per thread: the 2^16- and 2^17-point splits
        switch (d1.logL * 16 + d2.logL) {
        case 8 * 16 + 8: return launch_cluster_k<F, 8, 8, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
        case 7 * 16 + 9: return launch_cluster_k<F, 7, 9, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
        case 9 * 16 + 7: return launch_cluster_k<F, 9, 7, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
        case 8 * 16 + 9: return launch_cluster_k<F, 8, 9, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
        case 9 * 16 + 8: return launch_cluster_k<F, 9, 8, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
        default: return cudaErrorNotSupported;
        }
    }
    switch (d1.logL * 16 + d2.logL) {
    case 7 * 16 + 7: return launch_cluster_k<F, 7, 7>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 7 * 16 + 8: return launch_cluster_k<F, 7, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 8 * 16 + 7: return launch_cluster_k<F, 8, 7>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 7 * 16 + 9: return launch_cluster_k<F, 7, 9>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 8 * 16 + 8: return launch_cluster_k<F, 8, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 9 * 16 + 7: return launch_cluster_k<F, 9, 7>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 8 * 16 + 9: return launch_cluster_k<F, 8, 9>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    case 9 * 16 + 8: return launch_cluster_k<F, 9, 8>(a1, a2, xoff, xs, blocks, t, smem, log_k, s);
    default: return cudaErrorNotSupported;
    }
}

// Largest cluster (8 or 16) the device schedules for one 2^16-point cluster
// launch of this field (256 threads, its shared memory at 2^4 x 2^12 points).
template <class F>
int cluster_max_size_t() {
    auto kern = cluster_kernel<F, 8, 8, true>;
    if (cluster_attr<F, cluster_kernel<F, 8, 8, true>>() != cudaSuccess)
        return 8;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 80 * 1024;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 8;
    }
    return clusters > 0 ? 16 : 8;
}

template <class F>
cudaError_t preload_clusters_t() {
    const cudaError_t list[] = {
        cluster_attr<F, cluster_kernel<F, 7, 7, true>>(), cluster_attr<F, cluster_kernel<F, 7, 8, true>>(),
        cluster_attr<F, cluster_kernel<F, 8, 7, true>>(), cluster_attr<F, cluster_kernel<F, 7, 9, true>>(),
        cluster_attr<F, cluster_kernel<F, 8, 8, true>>(), cluster_attr<F, cluster_kernel<F, 9, 7, true>>(),
        cluster_attr<F, cluster_kernel<F, 8, 9, true>>(), cluster_attr<F, cluster_kernel<F, 9, 8, true>>(),
        cluster_attr<F, cluster_kernel<F, 8, 8, true, 8>>(), cluster_attr<F, cluster_kernel<F, 7, 9, true, 8>>(),
        cluster_attr<F, cluster_kernel<F, 9, 7, true, 8>>(), cluster_attr<F, cluster_kernel<F, 8, 9, true, 8>>(),
        cluster_attr<F, cluster_kernel<F, 9, 8, true, 8>>(),
    };
    for (cudaError_t e : list)
        if (e != cudaSuccess)
            return e;
    return cudaSuccess;
}

// ---- persistent batched launch (batch.cuh)
template <class F>
size_t batch_args_size_t() {
    return sizeof(TileArgs<F>);
}

// One item descriptor for a pass over transforms whose data pointers are in
// in_ptrs / out_ptrs (device arrays), `total` columns or rows in all.
template <class F>
void batch_args_fill_t(const PassDesc &d, uint32_t p, const void *tables, const unsigned long long *in_ptrs,
                       const unsigned long long *out_ptrs, uint64_t total, void *dst) {
    TileArgs<F> a;
    fill_args<F>(a, d, p, tables, nullptr, nullptr);
    a.in_ptrs = in_ptrs;
    a.out_ptrs = out_ptrs;
    a.total = total;
    memcpy(dst, &a, sizeof(a));
}

// Blocks per SM the persistent kernel is compiled for: 2 (64 registers per
// thread) unless STNTT_BATCH_MINB=1 selects the 128-register build.
inline int batch_minb() {
    static const int v = [] {
        const char *e = getenv("STNTT_BATCH_MINB");
        return (e && e[0] == '1') ? 1 : 2;
    }();
    return v;
}

template <class F>
cudaError_t batch_prepare_t(size_t smem, int *blocks_per_sm) {
    auto kern = batch_minb() == 1 ? batch_kernel<F, 1> : batch_kernel<F, 2>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess)
        return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kern, kBatchThreads, smem);
}

template <class F>
cudaError_t batch_launch_t(const void *args, const void *items, unsigned long long nitems, unsigned int *counters,
                           void *ctl, size_t smem, unsigned grid, unsigned spin_limit, cudaStream_t s) {
    auto kern = batch_minb() == 1 ? batch_kernel<F, 1> : batch_kernel<F, 2>;
    kern<<<grid, kBatchThreads, smem, s>>>(static_cast<const TileArgs<F> *>(args),
                                           static_cast<const BatchItem *>(items), nitems, counters,
                                           static_cast<BatchCtl *>(ctl), spin_limit);
    return cudaGetLastError();
}

// Load every tile and batch kernel of a field on the current device (CUDA
// loads kernel code lazily, at first use; a load in the middle of a serving
// loop stalls the device for a while), and set their shared-memory limits.
template <class F, int... LOGL>
cudaError_t preload_fixed_t(std::integer_sequence<int, LOGL...>) {
    cudaError_t e = cudaSuccess;
    ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_l<F, LOGL + 4>>() : e)), ...);
    ((e = (e == cudaSuccess && LOGL + 4 >= 6 ? tile_attr<F, tile_kernel_l<F, LOGL + 4, (LOGL + 4 >= 6)>>() : e)),
     ...);
    if constexpr (std::is_same_v<F, FieldU32L>) {
        ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_l<F, LOGL + 4, false, kU32MinBlocks>>() : e)), ...);
        ((e = (e == cudaSuccess && LOGL + 4 >= 6
                   ? tile_attr<F, tile_kernel_l<F, LOGL + 4, (LOGL + 4 >= 6), kU32MinBlocks>>()
                   : e)),
         ...);
    }
    return e;
}

template <class F, int... LOGL>
cudaError_t preload_fixed8_t(std::integer_sequence<int, LOGL...>) {
    cudaError_t e = cudaSuccess;
    ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_l<F, LOGL + 7, false, 1, 8>>() : e)), ...);
    ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_l<F, LOGL + 7, true, 1, 8>>() : e)), ...);
    return e;
}

template <class F>
cudaError_t preload_tiles_t() {
    const cudaError_t list[] = {
        tile_attr<F, tile_kernel<F, 2, 1>>(),        tile_attr<F, tile_kernel<F, 4, 2>>(),
        tile_attr<F, tile_kernel<F, 8, 3>>(),        tile_attr<F, tile_kernel<F, 16, 0>>(),
        tile_attr<F, tile_kernel<F, 16, 1>>(),       tile_attr<F, tile_kernel<F, 16, 2>>(),
        tile_attr<F, tile_kernel<F, 16, 3>>(),       tile_attr<F, tile_kernel<F, 32, 0>>(),
        tile_attr<F, tile_kernel<F, 32, 1>>(),       tile_attr<F, tile_kernel<F, 32, 2>>(),
        tile_attr<F, tile_kernel<F, 32, 3>>(),       tile_attr<F, tile_kernel<F, 2, 1, true>>(),
        tile_attr<F, tile_kernel<F, 4, 2, true>>(),  tile_attr<F, tile_kernel<F, 8, 3, true>>(),
        tile_attr<F, tile_kernel<F, 16, 0, true>>(), tile_attr<F, tile_kernel<F, 16, 1, true>>(),
        tile_attr<F, tile_kernel<F, 16, 2, true>>(), tile_attr<F, tile_kernel<F, 16, 3, true>>(),
        preload_fixed_t<F>(std::make_integer_sequence<int, 10>{}),
        preload_fixed8_t<F>(std::make_integer_sequence<int, 5>{}),
    };
    for (cudaError_t e : list)
        if (e != cudaSuccess)
            return e;
    if constexpr (IsPow2Field<F>::value) {
        return cudaSuccess;  // the batched kernel runs FieldGL (its launches mix directions)
    } else {
        int blocks = 0;
        return batch_prepare_t<F>(0, &blocks);
    }
}

// Twiddle entry from a residue (u32: Shoup pair {w, floor(w 2^32 / p)}).
template <class F>
__device__ __forceinline__ typename F::TW make_tw(uint64_t w, uint32_t p);
template <>
__device__ __forceinline__ uint2 make_tw<FieldU32>(uint64_t w, uint32_t p) {
    return make_uint2((uint32_t)w, (uint32_t)((w << 32) / p));
}
template <>
__device__ __forceinline__ uint64_t make_tw<FieldGL>(uint64_t w, uint32_t) {
    return w;
}

// The four-step twiddle of a column pass for every element of a sub-problem,
// in the data's own layout: out[pos * S + col] = lo[e mod 2^h] * hi[e >> h],
// e = col * pos < M.
template <class F>
__global__ void gen_four_step_kernel(typename F::TW *out, const typename F::TW *lo, const typename F::TW *hi,
                                     uint32_t h, uint32_t logS, uint64_t count, uint32_t p) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    const uint64_t e = (i >> logS) * (i & ((1ull << logS) - 1));
    const uint64_t a = F::tw_value(lo[e & ((1ull << h) - 1)]), b = F::tw_value(hi[e >> h]);
    uint64_t w;
    if constexpr (sizeof(typename F::T) == 8) {
        F f;
        f.p = p;
        w = f.mul(a, b);
    } else {
        w = a * b % p;
    }
    out[i] = make_tw<F>(w, p);
}

template <class F>
cudaError_t gen_four_step_t(void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS, uint64_t count,
                            uint32_t p, cudaStream_t s) {
    using TW = typename F::TW;
    const uint64_t blocks = (count + 255) / 256;
    if (!blocks)
        return cudaSuccess;
    gen_four_step_kernel<F><<<(unsigned)blocks, 256, 0, s>>>(static_cast<TW *>(out), static_cast<const TW *>(lo),
                                                             static_cast<const TW *>(hi), h, logS, count, p);
    return cudaGetLastError();
}

// out[i] = scale * base^i as twiddle entries
template <class F>
__global__ void gen_powers_kernel(typename F::TW *out, uint64_t count, uint64_t base, uint64_t scale, uint32_t p);

template <class F>
__global__ void pointwise_kernel(const typename F::T *a, const typename F::T *b, typename F::T *out, size_t count,
                                 uint32_t p) {
    F f;
    f.p = p;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
        out[i] = f.mul(a[i], b[i]);
}

template <class F>
__global__ void copy_scale_kernel(const typename F::T *in, typename F::T *out, size_t count, uint64_t scale_raw,
                                  uint32_t p) {
    F f;
    f.p = p;
    const typename F::TW w = to_tw<F>(scale_raw);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
        out[i] = f.mul_tw(in[i], w);
}

__device__ __forceinline__ uint64_t sm64_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t sm64_draw(uint64_t seed, uint64_t i, uint64_t attempt) {
    return sm64_mix(seed + 0x9E3779B97F4A7C15ull * (i + (attempt << 40) + 1ull));
}

inline unsigned grid_for(size_t count, unsigned threads) {
    size_t b = (count + threads - 1) / threads;
    if (b > 152u * 32u)
        b = 152u * 32u;
    return (unsigned)(b ? b : 1);
}

}  // namespace stntt
