// kernels_v_u32l.cu -- the vector-lines tile kernel (tile_v.cuh) over the
// 32-bit prime field with lazy reduction (p < 2^30: every findParams prime up
// to n = 2^26): four lines per thread, 16-byte accesses.
#include "kernels_v.cuh"

namespace stntt {

cudaError_t launch_tile_vec_u32l(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                                 uint64_t batch, cudaStream_t s) {
    return vlaunch::launch_tile_vec_t<FieldU32L>(d, p, tables, in, out, batch, s);
}

cudaError_t preload_vec_u32l() { return vlaunch::preload_v_t<FieldU32L>(); }

}  // namespace stntt
