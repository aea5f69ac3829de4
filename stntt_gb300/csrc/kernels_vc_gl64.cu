// kernels_vc_gl64.cu -- the vector-lines cluster pass (tile_vc.cuh) over
// Goldilocks, both directions (FieldGLF / FieldGLI).
#include "kernels_vc.cuh"

namespace stntt {

cudaError_t launch_tile_vc_gl64(const PassDesc &d, const void *tables, const void *in, void *out, uint64_t batch,
                                cudaStream_t s) {
    if (d.pow2 == 1)
        return vclaunch::launch_tile_vc_t<FieldGLF>(d, 0, tables, in, out, batch, s);
    if (d.pow2 == 2)
        return vclaunch::launch_tile_vc_t<FieldGLI>(d, 0, tables, in, out, batch, s);
    return cudaErrorNotSupported;
}

cudaError_t preload_vc_gl64() {
    const cudaError_t e = vclaunch::preload_vc_t<FieldGLF>();
    return e == cudaSuccess ? vclaunch::preload_vc_t<FieldGLI>() : e;
}

}  // namespace stntt
