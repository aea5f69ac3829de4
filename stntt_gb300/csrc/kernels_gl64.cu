// kernels_gl64.cu -- kernels over Goldilocks, p = 2^64 - 2^32 + 1.
#include "kernels_common.cuh"

namespace stntt {

template <>
__global__ void gen_powers_kernel<FieldGL>(uint64_t *out, uint64_t count, uint64_t base, uint64_t scale,
                                           uint32_t) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    FieldGL f;
    uint64_t r = scale, b = base;
    for (uint64_t e = i; e; e >>= 1) {
        if (e & 1)
            r = f.mul(r, b);
        b = f.mul(b, b);
    }
    out[i] = r;
}

__global__ void fill_uniform_gl64_kernel(uint64_t *out, size_t count, uint64_t seed) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        uint64_t x = 0;
        for (uint64_t a = 0;; ++a) {
            x = sm64_draw(seed, i, a);
            if (x < FieldGL::P)
                break;
        }
        out[i] = x;
    }
}

// The single-transform tile and cluster kernels are built per direction
// (FieldGLF / FieldGLI: shift-only internal twiddles) in kernels_gl64_f.cu and
// kernels_gl64_i.cu; every Goldilocks plan has one of the two roots
// (PassDesc::pow2). The batched kernel, whose launches mix directions, keeps
// FieldGL.
cudaError_t launch_tile_gl64f(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t, cudaStream_t,
                              const void *, int *);
cudaError_t launch_tile_gl64i(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t, cudaStream_t,
                              const void *, int *);
cudaError_t launch_cluster_gl64f(const PassDesc &, const PassDesc &, uint32_t, const void *, const void *, void *,
                                 uint64_t, uint32_t, uint32_t, size_t, uint32_t, cudaStream_t);
cudaError_t launch_cluster_gl64i(const PassDesc &, const PassDesc &, uint32_t, const void *, const void *, void *,
                                 uint64_t, uint32_t, uint32_t, size_t, uint32_t, cudaStream_t);
cudaError_t preload_gl64f();
cudaError_t preload_gl64i();

cudaError_t launch_tile_gl64(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                    uint64_t batch, cudaStream_t s, const void *in2, int *err) {
    if (d.pow2 == 1)
        return launch_tile_gl64f(d, p, tables, in, out, batch, s, in2, err);
    if (d.pow2 == 2)
        return launch_tile_gl64i(d, p, tables, in, out, batch, s, in2, err);
    return cudaErrorNotSupported;
}

cudaError_t gen_powers_gl64(void *out, uint64_t count, uint64_t base, uint64_t scale, cudaStream_t s) {
    const unsigned threads = 256;
    const uint64_t blocks = (count + threads - 1) / threads;
    if (!blocks)
        return cudaSuccess;
    gen_powers_kernel<FieldGL><<<(unsigned)blocks, threads, 0, s>>>(static_cast<uint64_t *>(out), count, base, scale,
                                                                    0);
    return cudaGetLastError();
}

cudaError_t pointwise_gl64(const void *a, const void *b, void *out, size_t count, cudaStream_t s) {
    pointwise_kernel<FieldGL><<<grid_for(count, 256), 256, 0, s>>>(
        static_cast<const uint64_t *>(a), static_cast<const uint64_t *>(b), static_cast<uint64_t *>(out), count, 0);
    return cudaGetLastError();
}

cudaError_t fill_uniform_gl64(void *out, size_t count, uint64_t seed, cudaStream_t s) {
    fill_uniform_gl64_kernel<<<grid_for(count, 256), 256, 0, s>>>(static_cast<uint64_t *>(out), count, seed);
    return cudaGetLastError();
}

cudaError_t copy_scale_gl64(const void *in, void *out, size_t count, uint64_t scale_tw, cudaStream_t s) {
    copy_scale_kernel<FieldGL><<<grid_for(count, 256), 256, 0, s>>>(static_cast<const uint64_t *>(in),
                                                                    static_cast<uint64_t *>(out), count, scale_tw, 0);
    return cudaGetLastError();
}

size_t batch_args_size_gl64() { return batch_args_size_t<FieldGL>(); }
void batch_args_fill_gl64(const PassDesc &d, uint32_t p, const void *tables, const unsigned long long *in_ptrs,
                         const unsigned long long *out_ptrs, uint64_t total, void *dst) {
    batch_args_fill_t<FieldGL>(d, p, tables, in_ptrs, out_ptrs, total, dst);
}
cudaError_t batch_prepare_gl64(size_t smem, int *blocks_per_sm) { return batch_prepare_t<FieldGL>(smem, blocks_per_sm); }
cudaError_t batch_launch_gl64(const void *args, const void *items, unsigned long long nitems, unsigned int *counters,
                             void *ctl, size_t smem, unsigned grid, unsigned spin_limit, cudaStream_t s) {
    return batch_launch_t<FieldGL>(args, items, nitems, counters, ctl, smem, grid, spin_limit, s);
}

}  // namespace stntt

// ---- integer throughput probe ------------------------------------------------
// The tile kernel's arithmetic without its memory traffic: every thread runs
// the radix-16 step (15 twiddle products, then the 16-point DIF network whose
// 17 internal twiddles are shifts, as in the tile kernels: dft_reg over
// FieldGLF) on 16 register values, `reps` times, and writes one checksum.
// Measures the Goldilocks butterfly rate this GPU sustains: the integer
// roofline the NTT kernels are compared with.
namespace stntt {

__global__ void __launch_bounds__(256) gl_butterfly_probe(uint64_t *out, int reps, uint64_t w1, uint64_t w2,
                                                          uint64_t w3) {
    FieldGLF f;
    uint64_t x[16];
    uint64_t seed = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * 0x9E3779B97F4A7C15ull + 1;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        seed = seed * 6364136223846793005ull + 1442695040888963407ull;
        x[i] = seed >> 1;  // < 2^63 < p
    }
    const uint64_t w[8] = {1, w1, w2, w3, w1 ^ 5, w2 ^ 7, w3 ^ 9, w1 ^ 11};
    for (int r = 0; r < reps; ++r) {
#pragma unroll
        for (int i = 1; i < 16; ++i)
            x[i] = f.mul(x[i], w[i & 7]);
        dft_reg<FieldGLF, 16>(f, x, w);
    }
    uint64_t acc = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i)
        acc ^= x[i] * (uint64_t)(i + 1);
    out[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

cudaError_t launch_gl_probe(uint64_t *out, unsigned blocks, int reps, cudaStream_t s) {
    gl_butterfly_probe<<<blocks, 256, 0, s>>>(out, reps, 0x1234567890ABCDEFull % FieldGL::P,
                                               0xFEDCBA9876543210ull % FieldGL::P, 0x0F0F0F0F0F0F0F0Full);
    return cudaGetLastError();
}

cudaError_t preload_gl64() {
    cudaFuncAttributes at;
    cudaError_t e = preload_gl64f();
    if (e == cudaSuccess)
        e = preload_gl64i();
    int blocks = 0;
    if (e == cudaSuccess)
        e = batch_prepare_t<FieldGL>(0, &blocks);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, gen_powers_kernel<FieldGL>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, gen_four_step_kernel<FieldGL>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, pointwise_kernel<FieldGL>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, copy_scale_kernel<FieldGL>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, fill_uniform_gl64_kernel);
    return e;
}

cudaError_t gen_four_step_gl64(void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS, uint64_t count,
                           uint32_t p, cudaStream_t s) {
    return gen_four_step_t<FieldGL>(out, lo, hi, h, logS, count, p, s);
}

cudaError_t launch_cluster_gl64(const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                                const void *in, void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem,
                                uint32_t log_k, cudaStream_t s) {
    if (d1.pow2 == 1 && d2.pow2 == 1)
        return launch_cluster_gl64f(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
    if (d1.pow2 == 2 && d2.pow2 == 2)
        return launch_cluster_gl64i(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
    return cudaErrorNotSupported;
}

}  // namespace stntt
