// kernels_tma_u32l.cu -- the TMA-staged tile kernel (tma.cuh) over the 32-bit
// prime field with lazy reduction (p < 2^30).
#include "tma_launch.cuh"

namespace stntt {

cudaError_t launch_tma_u32l(const PassDesc &d, const TileArgs<FieldU32L> &a, uint64_t batch, uint64_t tiles,
                            int *err, cudaStream_t s) {
    return launch_tma_t<FieldU32L>(d, a, batch, tiles, err, s);
}

cudaError_t preload_tma_u32l() { return preload_tma_t<FieldU32L>(std::make_integer_sequence<int, 6>{}); }

}  // namespace stntt
