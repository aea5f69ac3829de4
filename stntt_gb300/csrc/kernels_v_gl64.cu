// kernels_v_gl64.cu -- the vector-lines tile kernel (tile_v.cuh) over
// Goldilocks, forward transforms: two lines per thread, 16-byte accesses,
// internal twiddles as shifts (FieldGLF, w_16 = 2^156).
#include "kernels_v.cuh"

namespace stntt {

cudaError_t launch_tile_vec_gl64f(const PassDesc &d, const void *tables, const void *in, void *out, uint64_t batch,
                                  cudaStream_t s) {
    return vlaunch::launch_tile_vec_t<FieldGLF>(d, 0, tables, in, out, batch, s);
}

cudaError_t preload_vec_gl64f() { return vlaunch::preload_v_t<FieldGLF>(); }

}  // namespace stntt
