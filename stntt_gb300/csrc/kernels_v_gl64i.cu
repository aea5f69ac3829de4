// kernels_v_gl64i.cu -- the vector-lines tile kernel (tile_v.cuh) over
// Goldilocks, inverse transforms (FieldGLI, w_16 = 2^36); a file of its own so
// that the two directions compile in parallel.
#include "kernels_v.cuh"

namespace stntt {

cudaError_t launch_tile_vec_gl64i(const PassDesc &d, const void *tables, const void *in, void *out, uint64_t batch,
                                  cudaStream_t s) {
    return vlaunch::launch_tile_vec_t<FieldGLI>(d, 0, tables, in, out, batch, s);
}

cudaError_t preload_vec_gl64i() { return vlaunch::preload_v_t<FieldGLI>(); }

}  // namespace stntt
