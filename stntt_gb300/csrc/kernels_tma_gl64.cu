// kernels_tma_gl64.cu -- the TMA-staged tile kernel (tma.cuh) over Goldilocks,
// and the self-test of its bounded wait.
#include "tma_launch.cuh"

namespace stntt {

cudaError_t launch_tma_gl64(const PassDesc &d, const TileArgs<FieldGL> &a, uint64_t batch, uint64_t tiles, int *err,
                            cudaStream_t s) {
    return launch_tma_t<FieldGL>(d, a, batch, tiles, err, s);
}

cudaError_t preload_tma_gl64() { return preload_tma_t<FieldGL>(std::make_integer_sequence<int, 6>{}); }

// One CTA that issues no copy: its first wait polls spin_limit times, then
// sets *err and the CTA returns. It reads no memory besides its own shared
// memory (no tile is ever processed), so its arguments can stay empty.
cudaError_t launch_tma_selftest(int *err, uint32_t spin_limit, cudaStream_t s) {
    if (!err)
        return cudaErrorInvalidValue;
    TileArgs<FieldGL> a = {};
    a.logL = 8;
    a.logC = 1;
    a.cs = 272;
    TmaArgs t = {};
    t.ntiles = 1;
    t.stage_elems = 512;
    t.box_bytes = 4096;
    t.nbox = 1;
    t.spin_limit = spin_limit;
    t.skip_issue = 1;
    t.bar_off = (512 + 2 * 272) * 8;
    t.err = err;
    CUtensorMap tm;
    memset(&tm, 0, sizeof(tm));
    constexpr auto kern = tile_kernel_tma<FieldGL, 8, kModeRow, false>;
    cudaError_t e = tile_attr<FieldGL, kern>();
    if (e != cudaSuccess)
        return e;
    kern<<<1, 32, t.bar_off + 16, s>>>(a, tm, t);
    return cudaGetLastError();
}

}  // namespace stntt
