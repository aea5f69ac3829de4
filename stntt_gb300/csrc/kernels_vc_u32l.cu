// kernels_vc_u32l.cu -- the vector-lines cluster pass (tile_vc.cuh) over the
// lazy 32-bit field (p < 2^30).
#include "kernels_vc.cuh"

namespace stntt {

cudaError_t launch_tile_vc_u32l(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                                uint64_t batch, cudaStream_t s) {
    return vclaunch::launch_tile_vc_t<FieldU32L>(d, p, tables, in, out, batch, s);
}

cudaError_t preload_vc_u32l() { return vclaunch::preload_vc_t<FieldU32L>(); }

}  // namespace stntt
