// kernels_vc.cuh -- launch checks and launchers of the vector-lines cluster
// pass (tile_vc.cuh), instantiated per field by kernels_vc_gl64.cu and
// kernels_vc_u32l.cu.
#pragma once
#include "kernels_v.cuh"
#include "tile_vc.cuh"

namespace stntt {

namespace vclaunch {

using vlaunch::aligned16;
using vlaunch::vlines;

template <class F, int LOGL, int LOGG, bool COL, int FULL4>
cudaError_t launch_vc(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    constexpr int LOG1 = (LOGL + 1) / 2, LOGK = 3;
    constexpr auto kern = tile_kernel_vc<F, vlines<F>(), LOGL, LOG1, LOGG, LOGK, COL, FULL4>;
    cudaError_t e = vlaunch::vattr<F, kern>();
    if (e != cudaSuccess)
        return e;
    constexpr unsigned threads = vc_threads<LOGL, LOG1, LOGG, LOGK, vlines<F>()>();
    if (d.vsmem > 200 * 1024 || threads != d.vthreads || d.vlog1 != (uint32_t)LOG1 || d.vcl != (uint32_t)LOGK)
        return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = d.vsmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1u << LOGK;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    // programmatic dependent launch for calls of at least 2^22 elements (see pdl_min_elems)
    cfg.numAttrs = (a.total << d.logL) >= pdl_min_elems() ? 2 : 1;
    e = cudaLaunchKernelEx(&cfg, kern, a);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

template <class F, int LOGL, int LOGG>
cudaError_t launch_vc_mode(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    if (d.mode == kModeRow)
        return launch_vc<F, LOGL, LOGG, false, 0>(d, a, blocks, s);
    if constexpr (sizeof(typename F::T) == 4) {
        if (a.tw4_mont)
            return launch_vc<F, LOGL, LOGG, true, 2>(d, a, blocks, s);
    }
    if (a.tw4_full)
        return launch_vc<F, LOGL, LOGG, true, 1>(d, a, blocks, s);
    return launch_vc<F, LOGL, LOGG, true, 0>(d, a, blocks, s);
}

template <class F, int LOGL>
cudaError_t launch_vc_g(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    switch (d.vlogG) {
    case 2: return launch_vc_mode<F, LOGL, 2>(d, a, blocks, s);
    case 3: return launch_vc_mode<F, LOGL, 3>(d, a, blocks, s);
    default: return cudaErrorNotSupported;
    }
}

// Checks as launch_tile_vec_t; blocks = tiles * 8 (one cluster per tile).
template <class F>
cudaError_t launch_tile_vc_t(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                             uint64_t batch, cudaStream_t s) {
    constexpr uint32_t V = vlines<F>();
    if (!d.vcl || d.vec != V || d.vE != 8 || d.do_scale || d.logL >= d.logN || !aligned16(in) || !aligned16(out) ||
        !aligned16(tables))
        return cudaErrorNotSupported;
    const uint32_t C = V << d.vlogG;
    if (d.mode == kModeCol ? (1ull << d.logS) % C != 0 : (1ull << (d.logN - d.logL)) % C != 0)
        return cudaErrorNotSupported;
    TileArgs<F> a;
    fill_args<F>(a, d, p, tables, in, out);
    if ((a.tw4_full && !aligned16(a.tw4_full)) || (a.tw4_mont && !aligned16(a.tw4_mont)))
        return cudaErrorNotSupported;
    a.total = batch << (d.logN - d.logL);
    const uint64_t blocks = (a.total / C) << d.vcl;
    if (blocks == 0)
        return cudaSuccess;
    if (blocks > 0x7fffffffull)
        return cudaErrorInvalidConfiguration;
    switch (d.logL) {
    case 11: return launch_vc_g<F, 11>(d, a, blocks, s);
    case 12: return launch_vc_g<F, 12>(d, a, blocks, s);
    case 13: return launch_vc_g<F, 13>(d, a, blocks, s);
    default: return cudaErrorNotSupported;
    }
}

template <class F, int LOGL, int LOGG>
cudaError_t preload_vc_lg() {
    constexpr int LOG1 = (LOGL + 1) / 2, LOGK = 3, V = vlines<F>();
    constexpr uint32_t threads = vc_threads<LOGL, LOG1, LOGG, LOGK, V>();
    constexpr uint32_t regs = sizeof(typename F::T) == 8 ? 80 : 64;
    if constexpr (threads > 1024 || threads * regs > 65536) {
        return cudaSuccess;  // a shape the host never picks (shape_pass_vc)
    } else {
        cudaError_t e = vlaunch::vattr<F, tile_kernel_vc<F, V, LOGL, LOG1, LOGG, LOGK, false, 0>>();
        if (e == cudaSuccess)
            e = vlaunch::vattr<F, tile_kernel_vc<F, V, LOGL, LOG1, LOGG, LOGK, true, 0>>();
        if (e == cudaSuccess)
            e = vlaunch::vattr<F, tile_kernel_vc<F, V, LOGL, LOG1, LOGG, LOGK, true, 1>>();
        if constexpr (sizeof(typename F::T) == 4) {
            if (e == cudaSuccess)
                e = vlaunch::vattr<F, tile_kernel_vc<F, V, LOGL, LOG1, LOGG, LOGK, true, 2>>();
        }
        return e;
    }
}

template <class F>
cudaError_t preload_vc_t() {
    const cudaError_t list[] = {preload_vc_lg<F, 11, 2>(), preload_vc_lg<F, 11, 3>(), preload_vc_lg<F, 12, 2>(),
                                preload_vc_lg<F, 12, 3>(), preload_vc_lg<F, 13, 2>(), preload_vc_lg<F, 13, 3>()};
    for (cudaError_t e : list)
        if (e != cudaSuccess)
            return e;
    return cudaSuccess;
}

}  // namespace vclaunch

}  // namespace stntt
