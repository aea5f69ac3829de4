// kernels_gl64_i.cu -- the tile and cluster kernels over Goldilocks for
// inverse transforms (FieldGLI, w_16 = 2^36: internal twiddles as shifts); the
// two directions compile in parallel.
#include "kernels_common.cuh"

namespace stntt {

cudaError_t launch_tile_gl64i(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                              uint64_t batch, cudaStream_t s, const void *in2, int *err) {
    return launch_tile_t<FieldGLI>(d, p, tables, in, out, batch, s, in2, err);
}

cudaError_t launch_cluster_gl64i(const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                                 const void *in, void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem,
                                 uint32_t log_k, cudaStream_t s) {
    return launch_cluster_t<FieldGLI>(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
}

cudaError_t preload_gl64i() {
    const cudaError_t e = preload_tiles_t<FieldGLI>();
    return e == cudaSuccess ? preload_clusters_t<FieldGLI>() : e;
}

}  // namespace stntt
