// kernels_u32.cu -- kernels over the reference's per-size 32-bit prime field.
#include "../../include/stntt.h"
#include "kernels_common.cuh"

namespace stntt {

template <>
__global__ void gen_powers_kernel<FieldU32>(uint2 *out, uint64_t count, uint64_t base, uint64_t scale, uint32_t p) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    uint64_t r = scale % p, b = base % p;
    for (uint64_t e = i; e; e >>= 1) {
        if (e & 1)
            r = r * b % p;
        b = b * b % p;
    }
    out[i] = make_uint2((uint32_t)r, (uint32_t)((r << 32) / p));
}

__global__ void fill_uniform_u32_kernel(uint32_t *out, size_t count, uint64_t seed, uint32_t p) {
    const uint64_t limit = (1ull << 32) - ((1ull << 32) % p);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        uint64_t x = 0;
        for (uint64_t a = 0;; ++a) {
            x = sm64_draw(seed, i, a) >> 32;
            if (x < limit)
                break;
        }
        out[i] = (uint32_t)(x % p);
    }
}

// One radix-2 Stockham DIF stage (ntt_cpu.cpp:66-79). Butterfly m < n/2:
// l = v[m], r = v[m + n/2], J = 2^stage, s = m >> stage, j = m mod J,
// y[2sJ + j] = l + r, y[(2s+1)J + j] = w_(J s) (l - r).
__device__ __forceinline__ int32_t ref_modulo(int32_t x, int32_t mod) {
    int32_t r = x % mod;  // truncates toward zero, as in C++
    return r >= 0 ? r : r + mod;
}

__global__ void stage_u32_kernel(const uint32_t *in, uint32_t *out, const void *tw, uint32_t log_n, uint32_t stage,
                                 uint32_t p, int wrap, uint64_t total) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total)
        return;
    const uint64_t half = 1ull << (log_n - 1);
    const uint64_t b = gid >> (log_n - 1), m = gid & (half - 1);
    const uint64_t base = b << log_n;
    const uint64_t J = 1ull << stage, s = m >> stage, j = m & (J - 1);
    const uint64_t o0 = base + 2 * s * J + j, o1 = o0 + J;
    if (wrap) {
        // the reference's int32 arithmetic: the product wraps modulo 2^32
        const int32_t *tw32 = static_cast<const int32_t *>(tw);
        const int32_t l = (int32_t)in[base + m], r = (int32_t)in[base + m + half];
        const int32_t w = tw32[J * s];
        const int32_t md = (int32_t)p;
        out[o0] = (uint32_t)ref_modulo(l + r, md);
        const int32_t d = ref_modulo(l - r, md);
        out[o1] = (uint32_t)ref_modulo((int32_t)((uint32_t)w * (uint32_t)d), md);
    } else {
        FieldU32 f;
        f.p = p;
        const uint2 w = static_cast<const uint2 *>(tw)[J * s];
        const uint32_t l = in[base + m], r = in[base + m + half];
        out[o0] = f.add(l, r);
        out[o1] = f.mul_tw(f.sub(l, r), w);
    }
}

cudaError_t launch_stage_u32(const void *in, void *out, const void *tw, uint32_t log_n, uint32_t stage, uint32_t p,
                             int wrap, uint64_t batch, cudaStream_t s) {
    const uint64_t total = batch << (log_n - 1);
    const unsigned threads = 256;
    const uint64_t blocks = (total + threads - 1) / threads;
    if (blocks == 0)
        return cudaSuccess;
    stage_u32_kernel<<<(unsigned)blocks, threads, 0, s>>>(static_cast<const uint32_t *>(in),
                                                           static_cast<uint32_t *>(out), tw, log_n, stage, p, wrap,
                                                           total);
    return cudaGetLastError();
}

cudaError_t launch_tile_u32(const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                    uint64_t batch, cudaStream_t s, const void *in2, int *err) {
    return launch_tile_t<FieldU32>(d, p, tables, in, out, batch, s, in2, err);
}

cudaError_t gen_powers_u32(void *out, uint64_t count, uint64_t base, uint64_t scale, uint32_t p, cudaStream_t s) {
    const unsigned threads = 256;
    const uint64_t blocks = (count + threads - 1) / threads;
    if (!blocks)
        return cudaSuccess;
    gen_powers_kernel<FieldU32><<<(unsigned)blocks, threads, 0, s>>>(static_cast<uint2 *>(out), count, base, scale,
                                                                     p);
    return cudaGetLastError();
}

cudaError_t pointwise_u32(const void *a, const void *b, void *out, size_t count, uint32_t p, cudaStream_t s) {
    pointwise_kernel<FieldU32><<<grid_for(count, 256), 256, 0, s>>>(
        static_cast<const uint32_t *>(a), static_cast<const uint32_t *>(b), static_cast<uint32_t *>(out), count, p);
    return cudaGetLastError();
}

cudaError_t fill_uniform_u32(void *out, size_t count, uint64_t seed, uint32_t p, cudaStream_t s) {
    fill_uniform_u32_kernel<<<grid_for(count, 256), 256, 0, s>>>(static_cast<uint32_t *>(out), count, seed, p);
    return cudaGetLastError();
}

cudaError_t copy_scale_u32(const void *in, void *out, size_t count, uint64_t scale_tw, uint32_t p, cudaStream_t s) {
    copy_scale_kernel<FieldU32><<<grid_for(count, 256), 256, 0, s>>>(static_cast<const uint32_t *>(in),
                                                                     static_cast<uint32_t *>(out), count, scale_tw,
                                                                     p);
    return cudaGetLastError();
}

size_t batch_args_size_u32() { return batch_args_size_t<FieldU32>(); }
void batch_args_fill_u32(const PassDesc &d, uint32_t p, const void *tables, const unsigned long long *in_ptrs,
                         const unsigned long long *out_ptrs, uint64_t total, void *dst) {
    batch_args_fill_t<FieldU32>(d, p, tables, in_ptrs, out_ptrs, total, dst);
}
cudaError_t batch_prepare_u32(size_t smem, int *blocks_per_sm) { return batch_prepare_t<FieldU32>(smem, blocks_per_sm); }
cudaError_t batch_launch_u32(const void *args, const void *items, unsigned long long nitems, unsigned int *counters,
                             void *ctl, size_t smem, unsigned grid, unsigned spin_limit, cudaStream_t s) {
    return batch_launch_t<FieldU32>(args, items, nitems, counters, ctl, smem, grid, spin_limit, s);
}

// ---- findParams on the device ----------------------------------------------
// The reference's parameter search (src/ntt/ntt_util.cpp:10-49) for moduli
// below 2^32, in one CTA: the smallest prime p = k size + 1 >= min_mod
// (k >= 1; candidates tested blockDim.x at a time by trial division), the
// smallest generator g of Z_p^* (g^((p-1)/q) != 1 for every prime q | p - 1,
// tested blockDim.x at a time), root = g^((p-1)/size). out = {root, p,
// status}. Every loop ends: the prime search when the next candidate reaches
// 2^32 (status STNTT_EUNSUPPORTED), the generator search at g = p.
__device__ __forceinline__ uint64_t fp_powmod(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1)
            r = r * b % m;  // m < 2^32: products fit 64 bits
        b = b * b % m;
        e >>= 1;
    }
    return r;
}

__device__ bool fp_is_prime(uint64_t n) {
    if (n < 2)
        return n == 1;
    for (uint64_t x = 2; x * x <= n; ++x)
        if (n % x == 0)
            return false;
    return true;
}

__global__ void __launch_bounds__(256) find_params_kernel(uint64_t size, uint64_t min_mod, uint64_t *out) {
    __shared__ unsigned long long best;
    __shared__ uint64_t fac[32];
    __shared__ int nfac;
    constexpr uint64_t kLimit = 1ull << 32;
    const uint64_t k0 = max((min_mod - 1 + size - 1) / size, (uint64_t)1);
    uint64_t m = 0;
    for (uint64_t base = k0;; base += blockDim.x) {
        if (threadIdx.x == 0)
            best = ~0ull;
        __syncthreads();
        const uint64_t k = base + threadIdx.x;
        if (k < kLimit && k * size + 1 < kLimit && fp_is_prime(k * size + 1))
            atomicMin(&best, (unsigned long long)k);
        __syncthreads();
        const unsigned long long b = best;
        if (b != ~0ull) {
            m = b * size + 1;
            break;
        }
        if (base + blockDim.x >= kLimit || (base + blockDim.x) * size + 1 >= kLimit) {
            if (threadIdx.x == 0) {
                out[0] = 0;
                out[1] = 0;
                out[2] = STNTT_EUNSUPPORTED;
            }
            return;
        }
        __syncthreads();  // everyone has read `best` before it is reset
    }
    const uint64_t tot = m - 1;
    if (threadIdx.x == 0) {
        int nf = 0;
        uint64_t r = tot;
        for (uint64_t q = 2; q * q <= r; ++q)
            if (r % q == 0) {
                fac[nf++] = q;
                while (r % q == 0)
                    r /= q;
            }
        if (r > 1)
            fac[nf++] = r;
        nfac = nf;
        best = ~0ull;
    }
    __syncthreads();
    for (uint64_t base = 1; base < m; base += blockDim.x) {
        const uint64_t c = base + threadIdx.x;
        if (c < m && fp_powmod(c, tot, m) == 1 % m) {
            bool ok = true;
            for (int i = 0; i < nfac && ok; ++i)
                ok = fp_powmod(c, tot / fac[i], m) != 1;
            if (ok)
                atomicMin(&best, (unsigned long long)c);
        }
        __syncthreads();
        const unsigned long long b = best;
        if (b != ~0ull)
            break;
        __syncthreads();  // everyone has read `best` before the next candidates
    }
    if (threadIdx.x == 0) {
        const uint64_t g = best;
        out[0] = g == ~0ull ? 0 : fp_powmod(g, tot / size, m);
        out[1] = g == ~0ull ? 0 : m;
        out[2] = g == ~0ull ? STNTT_EUNSUPPORTED : STNTT_OK;
    }
}

cudaError_t launch_find_params(uint64_t size, uint64_t min_mod, uint64_t *out, cudaStream_t s) {
    find_params_kernel<<<1, 256, 0, s>>>(size, min_mod, out);
    return cudaGetLastError();
}

__global__ void gen_four_step_mont_kernel(uint32_t *out, const uint2 *lo, const uint2 *hi, uint32_t h, uint32_t logS,
                                          uint64_t count, uint32_t p, uint2 r32);

cudaError_t preload_u32() {
    cudaFuncAttributes at;
    cudaError_t e = preload_tiles_t<FieldU32>();
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, stage_u32_kernel);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, gen_powers_kernel<FieldU32>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, gen_four_step_kernel<FieldU32>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, pointwise_kernel<FieldU32>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, copy_scale_kernel<FieldU32>);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, fill_uniform_u32_kernel);
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&at, gen_four_step_mont_kernel);
    return e;
}

// out[pos * S + col] = w_M^(col * pos) * 2^32 mod p (Montgomery form), e = col * pos < M:
// two Shoup products (lo * hi, then by r32 = the Shoup pair of 2^32 mod p)
// instead of two 64-bit remainders (2^26 entries: 481 us per table before).
__global__ void gen_four_step_mont_kernel(uint32_t *out, const uint2 *lo, const uint2 *hi, uint32_t h, uint32_t logS,
                                          uint64_t count, uint32_t p, uint2 r32) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    FieldU32 f;
    f.p = p;
    const uint64_t e = (i >> logS) * (i & ((1ull << logS) - 1));
    const uint32_t w = f.mul_tw(lo[e & ((1ull << h) - 1)].x, hi[e >> h]);
    out[i] = f.mul_tw(w, r32);
}

cudaError_t gen_four_step_mont_u32(void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS, uint64_t count,
                                   uint32_t p, cudaStream_t s) {
    const uint64_t blocks = (count + 255) / 256;
    if (!blocks)
        return cudaSuccess;
    const uint32_t r = (uint32_t)((1ull << 32) % p);
    const uint2 r32 = make_uint2(r, (uint32_t)(((uint64_t)r << 32) / p));
    gen_four_step_mont_kernel<<<(unsigned)blocks, 256, 0, s>>>(static_cast<uint32_t *>(out),
                                                               static_cast<const uint2 *>(lo),
                                                               static_cast<const uint2 *>(hi), h, logS, count, p,
                                                               r32);
    return cudaGetLastError();
}

cudaError_t gen_four_step_u32(void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS, uint64_t count,
                           uint32_t p, cudaStream_t s) {
    return gen_four_step_t<FieldU32>(out, lo, hi, h, logS, count, p, s);
}

}  // namespace stntt
