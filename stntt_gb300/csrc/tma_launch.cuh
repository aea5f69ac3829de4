// tma_launch.cuh -- host side of the TMA-staged tile kernel (tma.cuh):
// whether a pass can use it, its tensor map, shared-memory layout and
// persistent grid. Included by kernels_tma_*.cu (one per field).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "kernels_common.cuh"
#include "tma.cuh"

namespace stntt {

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda); null when the driver does not provide it.
inline PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

struct TmaLaunch {
    CUtensorMap tm;
    TmaArgs t;
    size_t smem;
};

// Tensor map, shared-memory layout and arguments of one pass; false when the
// pass cannot run staged (tile length outside 2^7..2^12, fewer than 16 bytes
// of a column pass's row per tile, an input not 16-byte aligned, shared
// memory over the per-CTA budget, or a tensor map the driver refuses).
template <class F>
bool tma_setup(const PassDesc &d, const TileArgs<F> &a, uint64_t batch, uint64_t tiles, int *err, TmaLaunch &tl) {
    using T = typename F::T;
    constexpr uint64_t w = sizeof(T);
    if (!err || a.in2 || a.in_ptrs || d.E != 16 || d.logL < 7 || d.logL > 12)
        return false;
    if (reinterpret_cast<uintptr_t>(a.in) % 16 != 0)
        return false;
    auto encode = tmap_encoder();
    if (!encode)
        return false;
    const uint64_t L = 1ull << d.logL, C = 1ull << d.logC, n = 1ull << d.logN;
    const uint64_t Lb = std::min<uint64_t>(L, 256);
    cuuint64_t dims[4] = {1, 1, 1, 1}, strides[3] = {16, 16, 16};
    cuuint32_t box[4] = {1, 1, 1, 1}, es[4] = {1, 1, 1, 1};
    cuuint32_t rank;
    if (d.mode == kModeCol) {
        if (C * w < 16)
            return false;
        const uint64_t S = 1ull << d.logS, M = 1ull << d.logM;
        rank = 3;
        dims[0] = S;
        dims[1] = L;
        dims[2] = batch << (d.logN - d.logM);
        strides[0] = S * w;
        strides[1] = M * w;
        box[0] = (cuuint32_t)C;
        box[1] = (cuuint32_t)Lb;
        box[2] = 1;
    } else {
        const uint64_t n1 = 1ull << d.logN1, n2 = 1ull << d.logN2;
        if ((n1 * n2) << d.logL != n)
            return false;
        rank = 4;
        dims[0] = L;
        dims[1] = n1;
        dims[2] = n2;
        dims[3] = batch;
        strides[0] = n2 * L * w;
        strides[1] = L * w;
        strides[2] = n * w;
        const uint64_t b1 = std::min(C, n1), b2 = std::min(C / b1, n2);
        box[0] = (cuuint32_t)Lb;
        box[1] = (cuuint32_t)b1;
        box[2] = (cuuint32_t)b2;
        box[3] = (cuuint32_t)(C / (b1 * b2));
    }
    for (cuuint32_t i = 0; i < rank; ++i)
        if (dims[i] > (1ull << 32) || box[i] > 256)
            return false;
    for (cuuint32_t i = 0; i + 1 < rank; ++i)
        if (strides[i] % 16 != 0 || strides[i] >= (1ull << 40))
            return false;
    const uint64_t stage_bytes = C * L * w;
    const uint64_t bar_off = (stage_bytes + (uint64_t)d.cs * C * w + 7) & ~7ull;
    tl.smem = bar_off + 16;
    if (tl.smem > 200 * 1024)
        return false;
    const CUresult r = encode(&tl.tm, w == 8 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32, rank,
                              const_cast<T *>(a.in), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return false;
    tl.t.ntiles = tiles;
    tl.t.stage_elems = (uint32_t)(C * L);
    tl.t.box_bytes = (uint32_t)(C * Lb * w);
    tl.t.nbox = (uint32_t)(L / Lb);
    tl.t.spin_limit = kTmaSpinLimit;
    tl.t.skip_issue = 0;
    tl.t.bar_off = (uint32_t)bar_off;
    tl.t.err = err;
    return true;
}

// Resident CTAs of a kernel per SM for (threads, shared memory), cached.
inline int tma_occupancy(const void *kern, uint32_t threads, size_t smem) {
    struct Entry {
        const void *k;
        uint32_t threads;
        size_t smem;
        int dev, occ;
    };
    static std::mutex mu;
    static Entry cache[256];
    static int used = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    for (int i = 0; i < used; ++i)
        if (cache[i].k == kern && cache[i].threads == threads && cache[i].smem == smem && cache[i].dev == dev)
            return cache[i].occ;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, (int)threads, smem) != cudaSuccess) {
        cudaGetLastError();
        occ = 0;
    }
    if (used < 256)
        cache[used++] = {kern, threads, smem, dev, occ};
    return occ;
}

template <class F, int LOGL, int MODE, bool FULL4>
cudaError_t launch_tma_k(const PassDesc &d, const TileArgs<F> &a, const TmaLaunch &tl, cudaStream_t s) {
    constexpr auto kern = tile_kernel_tma<F, LOGL, MODE, FULL4>;
    cudaError_t e = tile_attr<F, kern>();
    if (e != cudaSuccess)
        return e;
    const int occ = tma_occupancy(reinterpret_cast<const void *>(kern), d.threads, tl.smem);
    if (occ <= 0)
        return cudaErrorNotSupported;
    // One tile per CTA: measured faster on GB300 than a persistent grid of
    // SMs x resident CTAs with next-tile prefetch (static or counter-claimed
    // tiles), whose staging buffer costs a resident CTA per SM. The kernel
    // takes either; a grid below the tile count prefetches.
    const uint64_t grid = tl.t.ntiles;
    kern<<<(unsigned)grid, d.threads, tl.smem, s>>>(a, tl.tm, tl.t);
    return cudaGetLastError();
}

template <class F, int LOGL>
cudaError_t launch_tma_l(const PassDesc &d, const TileArgs<F> &a, const TmaLaunch &tl, cudaStream_t s) {
    if (d.mode == kModeRow)
        return launch_tma_k<F, LOGL, kModeRow, false>(d, a, tl, s);
    if (a.tw4_full)
        return launch_tma_k<F, LOGL, kModeCol, true>(d, a, tl, s);
    return launch_tma_k<F, LOGL, kModeCol, false>(d, a, tl, s);
}

template <class F>
cudaError_t launch_tma_t(const PassDesc &d, const TileArgs<F> &a, uint64_t batch, uint64_t tiles, int *err,
                         cudaStream_t s) {
    TmaLaunch tl;
    if (!tma_setup<F>(d, a, batch, tiles, err, tl))
        return cudaErrorNotSupported;
    switch (d.logL) {
    case 7: return launch_tma_l<F, 7>(d, a, tl, s);
    case 8: return launch_tma_l<F, 8>(d, a, tl, s);
    case 9: return launch_tma_l<F, 9>(d, a, tl, s);
    case 10: return launch_tma_l<F, 10>(d, a, tl, s);
    case 11: return launch_tma_l<F, 11>(d, a, tl, s);
    case 12: return launch_tma_l<F, 12>(d, a, tl, s);
    default: return cudaErrorNotSupported;
    }
}

// Load every staged kernel of a field and raise its shared-memory limit.
template <class F, int... LOGL>
cudaError_t preload_tma_t(std::integer_sequence<int, LOGL...>) {
    (void)tmap_encoder();  // resolve the driver entry point outside any stream capture
    cudaError_t e = cudaSuccess;
    ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_tma<F, LOGL + 7, kModeRow, false>>() : e)), ...);
    ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_tma<F, LOGL + 7, kModeCol, false>>() : e)), ...);
    ((e = (e == cudaSuccess ? tile_attr<F, tile_kernel_tma<F, LOGL + 7, kModeCol, true>>() : e)), ...);
    return e;
}

}  // namespace stntt
