// kernels_gl64_f.cu -- the tile and cluster kernels over Goldilocks for
// forward transforms (FieldGLF, w_16 = 2^156: internal twiddles as shifts); the
// two directions compile in parallel.
#include "kernels_common.cuh"

namespace stntt {

cudaError_t launch_tile_gl64f(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                              uint64_t batch, cudaStream_t s, const void *in2, int *err) {
    return launch_tile_t<FieldGLF>(d, p, tables, in, out, batch, s, in2, err);
}

cudaError_t launch_cluster_gl64f(const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                                 const void *in, void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem,
                                 uint32_t log_k, cudaStream_t s) {
    return launch_cluster_t<FieldGLF>(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
}

cudaError_t preload_gl64f() {
    const cudaError_t e = preload_tiles_t<FieldGLF>();
    return e == cudaSuccess ? preload_clusters_t<FieldGLF>() : e;
}

int cluster_max_size() { return cluster_max_size_t<FieldGLF>(); }

}  // namespace stntt
