// kernels_u32l.cu -- tile and batched kernels over the 32-bit prime field with
// lazy reduction (FieldU32L, p < 2^30: every findParams prime up to n = 2^26).
#include "kernels_common.cuh"

namespace stntt {

cudaError_t launch_tile_u32l(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                    uint64_t batch, cudaStream_t s, const void *in2, int *err) {
    return launch_tile_t<FieldU32L>(d, p, tables, in, out, batch, s, in2, err);
}
cudaError_t batch_prepare_u32l(size_t smem, int *blocks_per_sm) { return batch_prepare_t<FieldU32L>(smem, blocks_per_sm); }
cudaError_t batch_launch_u32l(const void *args, const void *items, unsigned long long nitems, unsigned int *counters,
                              void *ctl, size_t smem, unsigned grid, unsigned spin_limit, cudaStream_t s) {
    static_assert(sizeof(TileArgs<FieldU32L>) == sizeof(TileArgs<FieldU32>), "same descriptor layout");
    return batch_launch_t<FieldU32L>(args, items, nitems, counters, ctl, smem, grid, spin_limit, s);
}

cudaError_t preload_u32l() {
    const cudaError_t e = preload_tiles_t<FieldU32L>();
    return e == cudaSuccess ? preload_clusters_t<FieldU32L>() : e;
}

cudaError_t launch_cluster_u32l(const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                                const void *in, void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem,
                                uint32_t log_k, cudaStream_t s) {
    return launch_cluster_t<FieldU32L>(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
}

}  // namespace stntt
