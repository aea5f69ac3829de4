// kernels_v.cuh -- launch checks and launchers of the vector-lines tile
// kernel (tile_v.cuh), instantiated per field by kernels_v_gl64.cu and
// kernels_v_u32l.cu.
#pragma once
#include <type_traits>

#include "kernels_common.cuh"
#include "tile_v.cuh"

namespace stntt {

namespace vlaunch {

template <class F>
constexpr int vlines() {
    return sizeof(typename F::T) == 4 ? 4 : 2;
}

template <class F, auto KERN>
cudaError_t vattr() {
    static bool set[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    if (!set[dev]) {
        e = cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess)
            return e;
        set[dev] = true;
    }
    return cudaSuccess;
}

template <class F, int E, int LOGL, int LOGG, bool COL, int FULL4>
cudaError_t launch_v(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    constexpr auto kern = tile_kernel_v<F, vlines<F>(), E, LOGL, LOGG, COL, FULL4>;
    cudaError_t e = vattr<F, kern>();
    if (e != cudaSuccess)
        return e;
    const unsigned threads = (1u << LOGG) * ((1u << LOGL) / E);
    if (d.vsmem > 200 * 1024 || threads != d.vthreads)
        return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = d.vsmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    // programmatic dependent launch for calls of at least 2^22 elements (see pdl_min_elems)
    cfg.numAttrs = (a.total << d.logL) >= pdl_min_elems() ? 1 : 0;
    e = cudaLaunchKernelEx(&cfg, kern, a);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

template <class F, int E, int LOGL, int LOGG>
cudaError_t launch_v_mode(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    if (d.mode == kModeRow)
        return launch_v<F, E, LOGL, LOGG, false, 0>(d, a, blocks, s);
    if constexpr (sizeof(typename F::T) == 4) {
        if (a.tw4_mont)
            return launch_v<F, E, LOGL, LOGG, true, 2>(d, a, blocks, s);
    }
    if (a.tw4_full)
        return launch_v<F, E, LOGL, LOGG, true, 1>(d, a, blocks, s);
    return launch_v<F, E, LOGL, LOGG, true, 0>(d, a, blocks, s);
}

// the thread limit of a (E, LOGL, LOGG) shape: 1024 up to 2^10-point tiles, 512 for wider ones
template <int E, int LOGL, int LOGG>
constexpr bool vfits() {
    return ((1u << LOGG) << LOGL) / E <= (LOGL <= 10 ? 1024u : 512u);
}

template <class F, int E, int LOGL>
cudaError_t launch_v_g(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    // line groups per CTA: 4 or 8 up to 2^10-point tiles; 1, 2 or 4 for the
    // wide tiles of two-pass plans (2^11 and 2^12 points), at most 512 threads
    // (at 1024 the 64-register limit spills the tile)
    if constexpr (LOGL <= 10) {
        switch (d.vlogG) {
        case 2:
            if constexpr (vfits<E, LOGL, 2>())
                return launch_v_mode<F, E, LOGL, 2>(d, a, blocks, s);
            return cudaErrorNotSupported;
        case 3:
            if constexpr (vfits<E, LOGL, 3>())
                return launch_v_mode<F, E, LOGL, 3>(d, a, blocks, s);
            return cudaErrorNotSupported;
        default: return cudaErrorNotSupported;
        }
    } else {
        switch (d.vlogG) {
        case 0:
            if constexpr (vfits<E, LOGL, 0>())
                return launch_v_mode<F, E, LOGL, 0>(d, a, blocks, s);
            return cudaErrorNotSupported;
        case 1:
            if constexpr (vfits<E, LOGL, 1>())
                return launch_v_mode<F, E, LOGL, 1>(d, a, blocks, s);
            return cudaErrorNotSupported;
        case 2:
            if constexpr (vfits<E, LOGL, 2>())
                return launch_v_mode<F, E, LOGL, 2>(d, a, blocks, s);
            return cudaErrorNotSupported;
        default: return cudaErrorNotSupported;
        }
    }
}

template <class F, int E>
cudaError_t launch_v_l(const PassDesc &d, const TileArgs<F> &a, uint64_t blocks, cudaStream_t s) {
    if constexpr (E == 4) {  // 4 points per line: the passes of single 2^18..2^22-point calls
        switch (d.logL) {
        case 9: return launch_v_g<F, E, 9>(d, a, blocks, s);
        case 10: return launch_v_g<F, E, 10>(d, a, blocks, s);
        case 11: return launch_v_g<F, E, 11>(d, a, blocks, s);
        default: return cudaErrorNotSupported;
        }
    } else {
        switch (d.logL) {
        case 7: return launch_v_g<F, E, 7>(d, a, blocks, s);
        case 8: return launch_v_g<F, E, 8>(d, a, blocks, s);
        case 9: return launch_v_g<F, E, 9>(d, a, blocks, s);
        case 10: return launch_v_g<F, E, 10>(d, a, blocks, s);
        case 11: return launch_v_g<F, E, 11>(d, a, blocks, s);
        case 12: return launch_v_g<F, E, 12>(d, a, blocks, s);
        default: return cudaErrorNotSupported;
        }
    }
}

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <class F>
cudaError_t launch_tile_vec_t(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                              uint64_t batch, cudaStream_t s) {
    constexpr uint32_t V = vlines<F>();
    if (!d.vec || d.vec != V || (d.vE != 4 && d.vE != 8 && d.vE != 16) || d.do_scale || d.logL >= d.logN || !aligned16(in) ||
        !aligned16(out) || !aligned16(tables))
        return cudaErrorNotSupported;
    const uint32_t C = V << d.vlogG;
    // C must divide the lines of one sub-problem (COL) or of one transform (ROW)
    if (d.mode == kModeCol ? (1ull << d.logS) % C != 0 : (1ull << (d.logN - d.logL)) % C != 0)
        return cudaErrorNotSupported;
    TileArgs<F> a;
    fill_args<F>(a, d, p, tables, in, out);
    if ((a.tw4_full && !aligned16(a.tw4_full)) || (a.tw4_mont && !aligned16(a.tw4_mont)))
        return cudaErrorNotSupported;
    a.total = batch << (d.logN - d.logL);
    const uint64_t blocks = a.total / C;
    if (blocks == 0)
        return cudaSuccess;
    if (blocks > 0x7fffffffull)
        return cudaErrorInvalidConfiguration;
    return d.vE == 4   ? launch_v_l<F, 4>(d, a, blocks, s)
           : d.vE == 8 ? launch_v_l<F, 8>(d, a, blocks, s)
                       : launch_v_l<F, 16>(d, a, blocks, s);
}

template <class F, int E, int LOGL, int LOGG>
cudaError_t preload_v_lg() {
    if constexpr (!vfits<E, LOGL, LOGG>())
        return cudaSuccess;  // a shape launch_v_g never launches
    cudaError_t e = vattr<F, tile_kernel_v<F, vlines<F>(), E, LOGL, LOGG, false, 0>>();
    if (e == cudaSuccess)
        e = vattr<F, tile_kernel_v<F, vlines<F>(), E, LOGL, LOGG, true, 0>>();
    if (e == cudaSuccess)
        e = vattr<F, tile_kernel_v<F, vlines<F>(), E, LOGL, LOGG, true, 1>>();
    if constexpr (sizeof(typename F::T) == 4) {
        if (e == cudaSuccess)
            e = vattr<F, tile_kernel_v<F, vlines<F>(), E, LOGL, LOGG, true, 2>>();
    }
    return e;
}

// the wide-tile shapes launch_v_g / launch_tile_vec_t can pick (else nothing to load)
template <class F, int E, int LOGL, int LOGG>
cudaError_t preload_v_wide() {
    return preload_v_lg<F, E, LOGL, LOGG>();
}

template <class F, int E>
cudaError_t preload_v_e() {
    const cudaError_t list[] = {preload_v_lg<F, E, 7, 2>(),  preload_v_lg<F, E, 7, 3>(),  preload_v_lg<F, E, 8, 2>(),
                                preload_v_lg<F, E, 8, 3>(),  preload_v_lg<F, E, 9, 2>(),  preload_v_lg<F, E, 9, 3>(),
                                preload_v_lg<F, E, 10, 2>(), preload_v_lg<F, E, 10, 3>(), preload_v_wide<F, E, 11, 0>(),
                                preload_v_wide<F, E, 11, 1>(), preload_v_wide<F, E, 11, 2>(), preload_v_wide<F, E, 12, 0>(),
                                preload_v_wide<F, E, 12, 1>(),  preload_v_wide<F, E, 12, 2>()};
    for (cudaError_t e : list)
        if (e != cudaSuccess)
            return e;
    return cudaSuccess;
}

template <class F>
cudaError_t preload_v_t() {
    const cudaError_t list[] = {preload_v_e<F, 16>(),        preload_v_e<F, 8>(),         preload_v_lg<F, 4, 9, 2>(),
                                preload_v_lg<F, 4, 9, 3>(),  preload_v_lg<F, 4, 10, 2>(), preload_v_wide<F, 4, 11, 0>()};
    for (cudaError_t e : list)
        if (e != cudaSuccess)
            return e;
    return cudaSuccess;
}

}  // namespace vlaunch

}  // namespace stntt
