// kernels_coop.cu -- the one-launch two-pass kernel (coop.cuh) for both
// fields: instantiations, residency check and the cooperative launch.
#include <map>
#include <mutex>
#include <tuple>

#include "coop.cuh"
#include "kernels_common.cuh"

namespace stntt {

namespace {

// CTAs of this kernel resident per SM at this shape (queried once per
// device, kernel, block size and shared memory), times the SM count.
int coop_capacity(const void *kern, unsigned threads, size_t smem) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, unsigned, size_t>, int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, kern, threads, smem);
    auto it = cache.find(key);
    if (it != cache.end())
        return it->second;
    int per_sm = 0, sms = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)threads, smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 0;
    }
    const int cap = per_sm * sms;
    cache[key] = cap;
    return cap;
}

template <class F, int LOG1, int LOG2, int E>
cudaError_t launch_coop_k(const TileArgs<F> &a1, const TileArgs<F> &a2, unsigned threads, size_t smem,
                          CoopBarrier *bar, int *err, cudaStream_t s) {
    auto kern = coop_kernel<F, LOG1, LOG2, E>;
    const int cap = coop_capacity(reinterpret_cast<const void *>(kern), threads, smem);
    const uint64_t tiles = std::max(a1.total >> a1.logC, a2.total >> a2.logC);
    if (cap <= 0 || threads > 512 || smem > 200 * 1024)
        return cudaErrorNotSupported;
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)cap);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a1, a2, bar, err, kTmaSpinLimit);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

// The (first, second) pass lengths instantiated: E = 8, tiles of 2^8..2^11
// points, transforms of 2^18..2^21 points (smaller two-pass transforms run as
// one thread-block-cluster launch, cluster.cuh).
template <class F>
cudaError_t launch_coop_t(const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables, const void *in,
                          void *ws, void *out, uint64_t batch, size_t smem, void *bar, int *err, cudaStream_t s) {
    if (d1.E != 8 || d2.E != 8 || d1.threads != d2.threads || d1.mode != kModeCol || d2.mode != kModeRow ||
        d1.full_off != ~0ull)
        return cudaErrorNotSupported;
    TileArgs<F> a1, a2;
    fill_args<F>(a1, d1, p, tables, in, ws);
    fill_args<F>(a2, d2, p, tables, ws, out);
    a1.total = batch << (d1.logN - d1.logL);
    a2.total = batch << (d2.logN - d2.logL);
    if ((a1.total & ((1ull << d1.logC) - 1)) || (a2.total & ((1ull << d2.logC) - 1)))
        return cudaErrorNotSupported;  // whole tiles only
    CoopBarrier *b = static_cast<CoopBarrier *>(bar);
    const unsigned t = d1.threads;
    switch (d1.logL * 16 + d2.logL) {
    case 8 * 16 + 10: return launch_coop_k<F, 8, 10, 8>(a1, a2, t, smem, b, err, s);
    case 9 * 16 + 9: return launch_coop_k<F, 9, 9, 8>(a1, a2, t, smem, b, err, s);
    case 10 * 16 + 8: return launch_coop_k<F, 10, 8, 8>(a1, a2, t, smem, b, err, s);
    case 8 * 16 + 11: return launch_coop_k<F, 8, 11, 8>(a1, a2, t, smem, b, err, s);
    case 9 * 16 + 10: return launch_coop_k<F, 9, 10, 8>(a1, a2, t, smem, b, err, s);
    case 10 * 16 + 9: return launch_coop_k<F, 10, 9, 8>(a1, a2, t, smem, b, err, s);
    case 11 * 16 + 8: return launch_coop_k<F, 11, 8, 8>(a1, a2, t, smem, b, err, s);
    case 9 * 16 + 11: return launch_coop_k<F, 9, 11, 8>(a1, a2, t, smem, b, err, s);
    case 10 * 16 + 10: return launch_coop_k<F, 10, 10, 8>(a1, a2, t, smem, b, err, s);
    case 11 * 16 + 9: return launch_coop_k<F, 11, 9, 8>(a1, a2, t, smem, b, err, s);
    case 10 * 16 + 11: return launch_coop_k<F, 10, 11, 8>(a1, a2, t, smem, b, err, s);
    case 11 * 16 + 10: return launch_coop_k<F, 11, 10, 8>(a1, a2, t, smem, b, err, s);
    default: return cudaErrorNotSupported;
    }
}

}  // namespace

cudaError_t launch_coop(int field, const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                        const void *in, void *ws, void *out, uint64_t batch, size_t smem, void *bar, int *err,
                        cudaStream_t s) {
    if (field == kFieldGL)
        return launch_coop_t<FieldGL>(d1, d2, p, tables, in, ws, out, batch, smem, bar, err, s);
    if (p < (1u << 30))
        return launch_coop_t<FieldU32L>(d1, d2, p, tables, in, ws, out, batch, smem, bar, err, s);
    return cudaErrorNotSupported;
}

}  // namespace stntt
