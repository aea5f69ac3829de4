/*
 * stntt_oracle.h -- CPU oracle for the stNTT hot path (TEST INFRASTRUCTURE).
 *
 * This library is the checker, not the product: only the test suite, the
 * smoke check and the CPU-baseline leg of bench.py may load it. The CUDA
 * library never links or calls it.
 *
 * It restates, in plain C, the reference's CPU algorithms for the forward and
 * inverse NTT (AlvaroPardoFente/stNTT, src/ntt/ntt_cpu.cpp and
 * src/ntt/ntt_util.cpp), with exact modular products:
 *   - field-exact Stockham DIF over the per-size 32-bit prime (u64 products)
 *   - the same loop with the reference's signed int32 wrap-around arithmetic
 *     ("ref-wrap"), bit-for-bit equal to the unmodified reference at every n
 *   - the same loop over Goldilocks p = 2^64 - 2^32 + 1 (u128 products)
 *   - O(n^2) schoolbook DFT and schoolbook polynomial products
 *   - the reference's test input generator (mt19937 + uniform_int{0,9})
 *
 * Pinning: tests/golden holds vectors produced by the unmodified reference
 * (compiled from its own sources by oracle/Makefile into oracle/_ref); the
 * CPU tests check this oracle against them.
 */
#ifndef STNTT_ORACLE_H
#define STNTT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_GL_P 0xFFFFFFFF00000001ull

/* ---- input generators ---------------------------------------------------- */
/* std::mt19937(seed) feeding libstdc++'s uniform_int_distribution<int>{lo,hi}
 * (src/util/rng.h:10-35). Writes n draws. */
void orc_mt19937_uniform_int(uint32_t seed, int32_t lo, int32_t hi, int32_t *out, size_t n);
/* splitmix64-seeded uniform residues in [0,p) by rejection. */
void orc_uniform_u32(uint64_t seed, uint32_t p, uint32_t *out, size_t n);
void orc_uniform_u64(uint64_t seed, uint64_t p, uint64_t *out, size_t n);

/* ---- number theory (src/ntt/ntt_util.cpp:10-93, ntt_util.h:66-95) -------- */
/* findParams(size, min_mod) -> (root, mod). Returns 0 on success. */
int orc_find_params(uint64_t size, uint64_t min_mod, uint64_t *root, uint64_t *mod);
uint64_t orc_pow_mod(uint64_t base, uint64_t e, uint64_t mod); /* mod < 2^63 */
uint64_t orc_gl_pow(uint64_t base, uint64_t e);
uint64_t orc_gl_mul(uint64_t a, uint64_t b);
uint64_t orc_gl_mul_slow(uint64_t a, uint64_t b);
/* omega_n = 7^((p-1)/n) for Goldilocks, n a power of two <= 2^32. */
uint64_t orc_gl_root(uint32_t log_n);

/* ---- Stockham DIF NTT, natural order in and out (ntt_cpu.cpp:46-85) ------- */
/* nsteps < 0: all log2(n) stages (the reference's std::nullopt). */
int orc_ntt_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod, int nsteps);
/* inverse: the same transform with root^-1, then scaled by n^-1. */
int orc_intt_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod);
int orc_ntt_gl64(uint64_t *vec, uint32_t n, uint64_t root, int nsteps);
int orc_intt_gl64(uint64_t *vec, uint32_t n, uint64_t root);
/* The reference's own int32 arithmetic, wrap-around included. */
int orc_ntt_ref_wrap(int32_t *vec, int32_t n, int32_t root, int32_t mod, int nsteps);
/* Batched: `batch` contiguous transforms; threads > 1 splits the batch. */
int orc_ntt_u32_batch(uint32_t *vec, uint32_t n, uint32_t batch, uint32_t root, uint32_t mod, int inverse,
                      int threads);
int orc_ntt_gl64_batch(uint64_t *vec, uint32_t n, uint32_t batch, int inverse, int threads);

/* ---- Cooley-Tukey NO->BO and Gentleman-Sande BO->NO (ntt_cpu.cpp:11-42, 130-164) */
int orc_ntt_ct_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod);
int orc_intt_gs_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod);

/* ---- schoolbook references ------------------------------------------------ */
void orc_dft_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t root, uint32_t mod);
void orc_dft_gl64(const uint64_t *in, uint64_t *out, uint32_t n, uint64_t root);
/* One DFT output X[k] = sum_j in[j] root^(j k), O(n): spot checks at sizes
 * where the full oracle is slow. */
uint32_t orc_dft_point_u32(const uint32_t *in, uint64_t n, uint32_t root, uint32_t mod, uint64_t k);
uint64_t orc_dft_point_gl64(const uint64_t *in, uint64_t n, uint64_t root, uint64_t k);
/* out[0..na+nb-2] = a * b (linear convolution mod p). */
void orc_polymul_u32(const uint32_t *a, size_t na, const uint32_t *b, size_t nb, uint32_t mod, uint32_t *out);
void orc_polymul_gl64(const uint64_t *a, size_t na, const uint64_t *b, size_t nb, uint64_t *out);

/* Cyclic convolution of length n via forward, element-wise product and
 * inverse (pwcNtt semantics, ntt_cpu.cpp:167-174). a <- a (*) b; b is
 * overwritten with its transform. */
int orc_cyclic_conv_u32(uint32_t *a, uint32_t *b, uint32_t n, uint32_t root, uint32_t mod);
int orc_cyclic_conv_gl64(uint64_t *a, uint64_t *b, uint32_t n);

/* ---- misc ------------------------------------------------------------------ */
uint64_t orc_fnv1a64(const void *data, size_t nbytes);

#ifdef __cplusplus
}
#endif
#endif
