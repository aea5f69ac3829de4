/*
 * stntt_oracle.c -- CPU oracle for the stNTT hot path (TEST INFRASTRUCTURE).
 *
 * Plain-C restatement of the reference algorithms (AlvaroPardoFente/stNTT).
 * Each function names the reference lines it follows. Only the test suite,
 * the smoke check and the CPU-baseline leg of bench.py use this file; the
 * CUDA library never links it.
 */
#include "stntt_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ========================================================================== */
/* input generators                                                            */
/* ========================================================================== */

/* MT19937 (Matsumoto & Nishimura 1998), as std::mt19937. */
typedef struct {
    uint32_t mt[624];
    int idx;
} orc_mt;

static void mt_seed(orc_mt *s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; ++i)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->idx = 624;
}

static uint32_t mt_next(orc_mt *s) {
    if (s->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = s->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u)
                v ^= 0x9908b0dfu;
            s->mt[i] = v;
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* util::Rng (src/util/rng.h:10-35): std::mt19937 + std::uniform_int_distribution<int>.
 * libstdc++ (GCC >= 11) downscales a 32-bit engine with Lemire's multiply-shift
 * method and a rejection threshold of (-range) % range. */
void orc_mt19937_uniform_int(uint32_t seed, int32_t lo, int32_t hi, int32_t *out, size_t n) {
    orc_mt s;
    mt_seed(&s, seed);
    uint32_t range = (uint32_t)(hi - lo) + 1u;
    uint32_t threshold = (uint32_t)(-range) % range;
    for (size_t i = 0; i < n; ++i) {
        uint64_t prod = (uint64_t)mt_next(&s) * range;
        uint32_t low = (uint32_t)prod;
        if (low < range) {
            while (low < threshold) {
                prod = (uint64_t)mt_next(&s) * range;
                low = (uint32_t)prod;
            }
        }
        out[i] = (int32_t)(prod >> 32) + lo;
    }
}

/* Counter-based splitmix64: draw (seed, i, attempt). The same definition is
 * implemented by the library's device generator and by numpy in the tests. */
static inline uint64_t sm64_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t sm64_draw(uint64_t seed, uint64_t i, uint64_t attempt) {
    return sm64_mix(seed + 0x9E3779B97F4A7C15ull * (i + (attempt << 40) + 1ull));
}

void orc_uniform_u32(uint64_t seed, uint32_t p, uint32_t *out, size_t n) {
    uint64_t limit = (1ull << 32) - ((1ull << 32) % p);
    for (size_t i = 0; i < n; ++i) {
        for (uint64_t a = 0;; ++a) {
            uint64_t x = sm64_draw(seed, i, a) >> 32;
            if (x < limit) {
                out[i] = (uint32_t)(x % p);
                break;
            }
        }
    }
}

void orc_uniform_u64(uint64_t seed, uint64_t p, uint64_t *out, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        for (uint64_t a = 0;; ++a) {
            uint64_t x = sm64_draw(seed, i, a);
            if (x < p) {
                out[i] = x;
                break;
            }
        }
    }
}

/* ========================================================================== */
/* number theory                                                               */
/* ========================================================================== */

uint64_t orc_pow_mod(uint64_t base, uint64_t e, uint64_t mod) {
    /* ntt_util.h:73-95 (non-negative exponent branch), exact with u128. */
    uint64_t r = 1 % mod;
    base %= mod;
    while (e) {
        if (e & 1)
            r = (uint64_t)(((u128)r * base) % mod);
        base = (uint64_t)(((u128)base * base) % mod);
        e >>= 1;
    }
    return r;
}

/* floor(sqrt(n)) by the reference's bit-by-bit method (ntt_util.cpp:75-86). */
static uint64_t isqrt(uint64_t n) {
    uint64_t i = 1, res = 0;
    while (i <= n / i)
        i *= 2;
    for (; i > 0; i /= 2)
        if ((res + i) <= n / (res + i) && (res + i) * (res + i) <= n)
            res += i;
    return res;
}

/* isPrime by trial division over [2, sqrt(n)] (ntt_util.h:66-70). */
static int is_prime(uint64_t n) {
    uint64_t e = isqrt(n);
    for (uint64_t x = 2; x <= e; ++x)
        if (n % x == 0)
            return 0;
    return 1;
}

/* uniquePrimeFactors (ntt_util.cpp:53-72). Returns the count. */
static int unique_prime_factors(uint64_t n, uint64_t *f) {
    int cnt = 0;
    uint64_t end = isqrt(n);
    for (uint64_t i = 2; i <= end; i++) {
        if (n % i == 0) {
            n /= i;
            f[cnt++] = i;
            while (n % i == 0)
                n /= i;
            end = isqrt(n);
        }
    }
    if (n > 1)
        f[cnt++] = n;
    return cnt;
}

/* isPrimitiveRoot (ntt_util.cpp:44-50). */
static int is_primitive_root(uint64_t val, uint64_t degree, uint64_t mod) {
    uint64_t f[64];
    int cnt = unique_prime_factors(degree, f);
    if (orc_pow_mod(val, degree, mod) != 1 % mod)
        return 0;
    for (int i = 0; i < cnt; ++i)
        if (orc_pow_mod(val, degree / f[i], mod) == 1)
            return 0;
    return 1;
}

/* findParams -> findModulus, findPrimitiveRoot, findGenerator (ntt_util.cpp:10-42).
 * Smallest prime mod = k*size + 1 >= min_mod, root = g^((mod-1)/size) with g
 * the smallest generator of the multiplicative group. */
int orc_find_params(uint64_t size, uint64_t min_mod, uint64_t *root, uint64_t *mod) {
    if (size == 0 || min_mod == 0)
        return -1;
    uint64_t start = (min_mod - 1 + size - 1) / size;
    if (start < 1)
        start = 1;
    uint64_t m = 0;
    for (uint64_t k = start;; ++k) {
        if (k > UINT64_MAX / size)
            return -2;
        uint64_t cand = k * size + 1;
        if (is_prime(cand)) {
            m = cand;
            break;
        }
    }
    uint64_t totient = m - 1, g = 0;
    for (uint64_t i = 1; i < m; ++i)
        if (is_primitive_root(i, totient, m)) {
            g = i;
            break;
        }
    if (g == 0)
        return -3;
    *mod = m;
    *root = orc_pow_mod(g, totient / size, m);
    return 0;
}

/* ---- Goldilocks ----------------------------------------------------------- */
/* a*b mod p via 2^64 = 2^32 - 1 and 2^96 = -1 (mod p); orc_gl_mul_slow is
 * the plain 128-bit remainder the tests compare it with. */
uint64_t orc_gl_mul(uint64_t a, uint64_t b) {
    const uint64_t EPS = 0xffffffffull;
    u128 x = (u128)a * b;
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    uint64_t hh = hi >> 32, hl = hi & EPS;
    uint64_t t = lo - hh;
    if (lo < hh)
        t -= EPS;
    uint64_t u = hl * EPS;
    uint64_t s = t + u;
    if (s < u)
        s += EPS;
    if (s >= ORC_GL_P)
        s -= ORC_GL_P;
    return s;
}
uint64_t orc_gl_mul_slow(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * b) % ORC_GL_P); }
/* canonical a, b < p */
static inline uint64_t gl_add(uint64_t a, uint64_t b) {
    uint64_t s = a + b;
    if (s < a || s >= ORC_GL_P) /* carry out of 2^64, or >= p: subtract p */
        s -= ORC_GL_P;
    return s;
}
static inline uint64_t gl_sub(uint64_t a, uint64_t b) { return a >= b ? a - b : a - b + ORC_GL_P; }
uint64_t orc_gl_pow(uint64_t base, uint64_t e) {
    uint64_t r = 1;
    base %= ORC_GL_P;
    while (e) {
        if (e & 1)
            r = orc_gl_mul(r, base);
        base = orc_gl_mul(base, base);
        e >>= 1;
    }
    return r;
}
uint64_t orc_gl_root(uint32_t log_n) {
    if (log_n > 32)
        return 0;
    return orc_gl_pow(7, (ORC_GL_P - 1) >> log_n);
}

static int log2_exact(uint64_t n) {
    if (n == 0 || (n & (n - 1)))
        return -1;
    int l = 0;
    while ((1ull << l) < n)
        ++l;
    return l;
}

/* ========================================================================== */
/* Stockham DIF, natural order in and out (ntt_cpu.cpp:46-85)                 */
/* ========================================================================== */

int orc_ntt_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod, int nsteps) {
    int steps = log2_exact(n);
    if (steps < 0 || mod < 2)
        return -1;
    uint32_t *y = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t *tw = (uint32_t *)malloc(sizeof(uint32_t) * (n / 2 + 1));
    if (!y || !tw) {
        free(y);
        free(tw);
        return -2;
    }
    /* pow_table[i] = root^i, i < n/2 (ntt_cpu.cpp:57-62), exact. */
    uint64_t t = 1;
    for (uint32_t i = 0; i < n / 2; ++i) {
        tw[i] = (uint32_t)t;
        t = t * root % mod;
    }
    if (nsteps >= 0)
        steps = nsteps;
    uint32_t *v = vec, *out = y;
    const uint32_t half = n / 2;
    for (int i = 0; i < steps; ++i) {
        uint32_t J = 1u << i;
        for (uint32_t s = 0; s < n / (2 * J); ++s) {
            uint64_t w = tw[J * s];
            for (uint32_t j = 0; j < J; ++j) {
                uint32_t l = v[s * J + j], r = v[s * J + j + half];
                uint32_t sum = (uint32_t)(((uint64_t)l + r) % mod);
                uint32_t diff = (uint32_t)(((uint64_t)l + mod - r % mod) % mod);
                out[2 * s * J + j] = sum;
                out[(2 * s + 1) * J + j] = (uint32_t)(w * diff % mod);
            }
        }
        uint32_t *tmp = v;
        v = out;
        out = tmp;
    }
    if (v != vec)
        memcpy(vec, v, sizeof(uint32_t) * n);
    free(y);
    free(tw);
    return 0;
}

int orc_intt_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod) {
    uint32_t rinv = (uint32_t)orc_pow_mod(root, mod - 2, mod);
    int rc = orc_ntt_u32(vec, n, rinv, mod, -1);
    if (rc)
        return rc;
    uint64_t ninv = orc_pow_mod(n % mod, mod - 2, mod);
    for (uint32_t i = 0; i < n; ++i)
        vec[i] = (uint32_t)(vec[i] * ninv % mod);
    return 0;
}

int orc_ntt_gl64(uint64_t *vec, uint32_t n, uint64_t root, int nsteps) {
    int steps = log2_exact(n);
    if (steps < 0)
        return -1;
    uint64_t *y = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
    uint64_t *tw = (uint64_t *)malloc(sizeof(uint64_t) * (n / 2 + 1));
    if (!y || !tw) {
        free(y);
        free(tw);
        return -2;
    }
    uint64_t t = 1;
    for (uint32_t i = 0; i < n / 2; ++i) {
        tw[i] = t;
        t = orc_gl_mul(t, root);
    }
    if (nsteps >= 0)
        steps = nsteps;
    for (uint32_t i = 0; i < n; ++i)
        if (vec[i] >= ORC_GL_P)
            vec[i] -= ORC_GL_P;
    uint64_t *v = vec, *out = y;
    const uint32_t half = n / 2;
    for (int i = 0; i < steps; ++i) {
        uint32_t J = 1u << i;
        for (uint32_t s = 0; s < n / (2 * J); ++s) {
            uint64_t w = tw[J * s];
            for (uint32_t j = 0; j < J; ++j) {
                uint64_t l = v[s * J + j], r = v[s * J + j + half];
                out[2 * s * J + j] = gl_add(l, r);
                out[(2 * s + 1) * J + j] = orc_gl_mul(w, gl_sub(l, r));
            }
        }
        uint64_t *tmp = v;
        v = out;
        out = tmp;
    }
    if (v != vec)
        memcpy(vec, v, sizeof(uint64_t) * n);
    free(y);
    free(tw);
    return 0;
}

int orc_intt_gl64(uint64_t *vec, uint32_t n, uint64_t root) {
    uint64_t rinv = orc_gl_pow(root, ORC_GL_P - 2);
    int rc = orc_ntt_gl64(vec, n, rinv, -1);
    if (rc)
        return rc;
    uint64_t ninv = orc_gl_pow(n, ORC_GL_P - 2);
    for (uint32_t i = 0; i < n; ++i)
        vec[i] = orc_gl_mul(vec[i], ninv);
    return 0;
}

/* The same loop with the reference's signed 32-bit arithmetic: products wrap
 * modulo 2^32 and '%' truncates toward zero, as in ntt_cpu.cpp:57-79 with
 * modulo() from ntt_util.cpp:88-93. Unsigned multiplies give the wrap without
 * relying on signed overflow. */
static inline int32_t wrap_mul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
static inline int32_t ref_modulo(int32_t x, int32_t mod) {
    int32_t r = x % mod;
    return r >= 0 ? r : r + mod;
}

int orc_ntt_ref_wrap(int32_t *vec, int32_t n, int32_t root, int32_t mod, int nsteps) {
    int steps = log2_exact((uint64_t)(uint32_t)n);
    if (n <= 0 || steps < 0 || mod < 2)
        return -1;
    int32_t *y = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t *tw = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n / 2 + 1));
    if (!y || !tw) {
        free(y);
        free(tw);
        return -2;
    }
    int32_t temp = 1;
    for (int32_t i = 0; i < n / 2; ++i) {
        tw[i] = temp;
        temp = wrap_mul(temp, root) % mod;
    }
    if (nsteps >= 0)
        steps = nsteps;
    int32_t *v = vec, *out = y;
    for (int i = 0; i < steps; ++i) {
        int32_t J = 1 << i;
        for (int32_t s = 0; s < n / (2 * J); ++s) {
            int32_t w = tw[J * s];
            for (int32_t j = 0; j < J; ++j) {
                int32_t l = v[s * J + j], r = v[s * J + j + n / 2];
                out[2 * s * J + j] = ref_modulo(l + r, mod);
                out[(2 * s + 1) * J + j] = ref_modulo(wrap_mul(w, ref_modulo(l - r, mod)), mod);
            }
        }
        int32_t *tmp = v;
        v = out;
        out = tmp;
    }
    if (v != vec)
        memcpy(vec, v, sizeof(int32_t) * (size_t)n);
    free(y);
    free(tw);
    return 0;
}

/* ---- batched, optionally threaded (ntt_cpu.cpp:87-90 loops sequentially) --- */
typedef struct {
    void *vec;
    uint32_t n, b0, b1;
    uint64_t root, mod;
    int inverse, gl;
    int rc;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *j = (batch_job *)arg;
    j->rc = 0;
    for (uint32_t b = j->b0; b < j->b1 && !j->rc; ++b) {
        if (j->gl) {
            uint64_t *v = (uint64_t *)j->vec + (size_t)b * j->n;
            j->rc = j->inverse ? orc_intt_gl64(v, j->n, j->root) : orc_ntt_gl64(v, j->n, j->root, -1);
        } else {
            uint32_t *v = (uint32_t *)j->vec + (size_t)b * j->n;
            j->rc = j->inverse ? orc_intt_u32(v, j->n, (uint32_t)j->root, (uint32_t)j->mod)
                               : orc_ntt_u32(v, j->n, (uint32_t)j->root, (uint32_t)j->mod, -1);
        }
    }
    return NULL;
}

static int run_batch(void *vec, uint32_t n, uint32_t batch, uint64_t root, uint64_t mod, int inverse, int gl,
                     int threads) {
    if (threads < 1)
        threads = 1;
    if ((uint32_t)threads > batch)
        threads = batch ? (int)batch : 1;
    batch_job jobs[256];
    pthread_t tid[256];
    if (threads > 256)
        threads = 256;
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (batch_job){vec, n, (uint32_t)((uint64_t)batch * t / threads),
                              (uint32_t)((uint64_t)batch * (t + 1) / threads), root, mod, inverse, gl, 0};
    }
    if (threads == 1) {
        batch_worker(&jobs[0]);
        return jobs[0].rc;
    }
    for (int t = 0; t < threads; ++t)
        pthread_create(&tid[t], NULL, batch_worker, &jobs[t]);
    int rc = 0;
    for (int t = 0; t < threads; ++t) {
        pthread_join(tid[t], NULL);
        if (jobs[t].rc)
            rc = jobs[t].rc;
    }
    return rc;
}

int orc_ntt_u32_batch(uint32_t *vec, uint32_t n, uint32_t batch, uint32_t root, uint32_t mod, int inverse,
                      int threads) {
    return run_batch(vec, n, batch, root, mod, inverse, 0, threads);
}

int orc_ntt_gl64_batch(uint64_t *vec, uint32_t n, uint32_t batch, int inverse, int threads) {
    int l = log2_exact(n);
    if (l < 0 || l > 32)
        return -1;
    return run_batch(vec, n, batch, orc_gl_root((uint32_t)l), ORC_GL_P, inverse, 1, threads);
}

/* ========================================================================== */
/* Cooley-Tukey (NO->BO) and Gentleman-Sande (BO->NO), field-exact             */
/* ========================================================================== */

static uint32_t bitrev(uint32_t x, int bits) {
    uint32_t y = 0;
    for (int i = 0; i < bits; ++i) {
        y = (y << 1) | (x & 1);
        x >>= 1;
    }
    return y;
}

/* nttCt (ntt_cpu.cpp:11-42): bit-reversed power table, natural in, bit-reversed out. */
int orc_ntt_ct_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod) {
    int levels = log2_exact(n);
    if (levels < 0)
        return -1;
    uint32_t *tw = (uint32_t *)malloc(sizeof(uint32_t) * (n / 2 + 1));
    if (!tw)
        return -2;
    uint64_t t = 1;
    for (uint32_t i = 0; i < n / 2; ++i) {
        tw[i] = (uint32_t)t;
        t = t * root % mod;
    }
    int tb = levels > 0 ? levels - 1 : 0;
    for (uint32_t i = 0; i < n / 2; ++i) {
        uint32_t j = bitrev(i, tb);
        if (j > i) {
            uint32_t x = tw[i];
            tw[i] = tw[j];
            tw[j] = x;
        }
    }
    for (uint32_t size = n; size >= 2; size /= 2) {
        uint32_t hs = size / 2, k = 0;
        for (uint32_t i = 0; i < n; i += size) {
            for (uint32_t j = i; j < i + hs; ++j) {
                uint64_t left = vec[j], right = (uint64_t)vec[j + hs] * tw[k] % mod;
                vec[j] = (uint32_t)((left + right) % mod);
                vec[j + hs] = (uint32_t)((left + mod - right) % mod);
            }
            k++;
        }
    }
    free(tw);
    return 0;
}

/* inttGs (ntt_cpu.cpp:130-164): bit-reversed root^-i table, then n^-1. */
int orc_intt_gs_u32(uint32_t *vec, uint32_t n, uint32_t root, uint32_t mod) {
    int levels = log2_exact(n);
    if (levels < 0)
        return -1;
    uint32_t *tw = (uint32_t *)malloc(sizeof(uint32_t) * (n / 2 + 1));
    if (!tw)
        return -2;
    uint64_t rinv = orc_pow_mod(root, mod - 2, mod), t = 1;
    for (uint32_t i = 0; i < n / 2; ++i) {
        tw[i] = (uint32_t)t;
        t = t * rinv % mod;
    }
    int tb = levels > 0 ? levels - 1 : 0;
    for (uint32_t i = 0; i < n / 2; ++i) {
        uint32_t j = bitrev(i, tb);
        if (j > i) {
            uint32_t x = tw[i];
            tw[i] = tw[j];
            tw[j] = x;
        }
    }
    for (uint32_t size = 2; size <= n; size *= 2) {
        uint32_t hs = size / 2, k = 0;
        for (uint32_t i = 0; i < n; i += size) {
            for (uint32_t j = i; j < i + hs; ++j) {
                uint64_t left = vec[j], right = vec[j + hs];
                vec[j] = (uint32_t)((left + right) % mod);
                vec[j + hs] = (uint32_t)((left + mod - right) % mod * tw[k] % mod);
            }
            k++;
        }
    }
    uint64_t ninv = orc_pow_mod(n % mod, mod - 2, mod);
    for (uint32_t i = 0; i < n; ++i)
        vec[i] = (uint32_t)(vec[i] * ninv % mod);
    free(tw);
    return 0;
}

/* ========================================================================== */
/* schoolbook references                                                       */
/* ========================================================================== */

void orc_dft_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t root, uint32_t mod) {
    uint64_t wk = 1; /* root^k */
    for (uint32_t k = 0; k < n; ++k) {
        uint64_t acc = 0, w = 1; /* w = root^(j*k) */
        for (uint32_t j = 0; j < n; ++j) {
            acc = (acc + (uint64_t)in[j] % mod * w) % mod;
            w = w * wk % mod;
        }
        out[k] = (uint32_t)acc;
        wk = wk * root % mod;
    }
}

void orc_dft_gl64(const uint64_t *in, uint64_t *out, uint32_t n, uint64_t root) {
    uint64_t wk = 1;
    for (uint32_t k = 0; k < n; ++k) {
        uint64_t acc = 0, w = 1;
        for (uint32_t j = 0; j < n; ++j) {
            acc = gl_add(acc, orc_gl_mul(in[j] % ORC_GL_P, w));
            w = orc_gl_mul(w, wk);
        }
        out[k] = acc;
        wk = orc_gl_mul(wk, root);
    }
}

uint32_t orc_dft_point_u32(const uint32_t *in, uint64_t n, uint32_t root, uint32_t mod, uint64_t k) {
    const uint64_t wk = orc_pow_mod(root, k % n, mod);
    uint64_t acc = 0, w = 1;
    for (uint64_t j = 0; j < n; ++j) {
        acc = (acc + (uint64_t)in[j] % mod * w) % mod;
        w = w * wk % mod;
    }
    return (uint32_t)acc;
}

uint64_t orc_dft_point_gl64(const uint64_t *in, uint64_t n, uint64_t root, uint64_t k) {
    const uint64_t wk = orc_gl_pow(root, k % n);
    uint64_t acc = 0, w = 1;
    for (uint64_t j = 0; j < n; ++j) {
        acc = gl_add(acc, orc_gl_mul(in[j] % ORC_GL_P, w));
        w = orc_gl_mul(w, wk);
    }
    return acc;
}

void orc_polymul_u32(const uint32_t *a, size_t na, const uint32_t *b, size_t nb, uint32_t mod, uint32_t *out) {
    if (!na || !nb)
        return;
    size_t no = na + nb - 1;
    for (size_t i = 0; i < no; ++i)
        out[i] = 0;
    for (size_t i = 0; i < na; ++i)
        for (size_t j = 0; j < nb; ++j)
            out[i + j] = (uint32_t)((out[i + j] + (uint64_t)a[i] * b[j]) % mod);
}

void orc_polymul_gl64(const uint64_t *a, size_t na, const uint64_t *b, size_t nb, uint64_t *out) {
    if (!na || !nb)
        return;
    size_t no = na + nb - 1;
    for (size_t i = 0; i < no; ++i)
        out[i] = 0;
    for (size_t i = 0; i < na; ++i)
        for (size_t j = 0; j < nb; ++j)
            out[i + j] = gl_add(out[i + j], orc_gl_mul(a[i], b[j]));
}

/* Cyclic convolution of length n through the transform, the semantics of
 * pwcNtt (ntt_cpu.cpp:167-174): forward transform of both inputs, element-wise
 * product (elemWiseMul, ntt_util.h:29-33, with exact products here), inverse
 * scaled by n^-1. The reference goes NO->BO->NO (nttCt / inttGs); natural
 * order on both sides gives the same result. a is overwritten with the
 * result, b with its transform. */
int orc_cyclic_conv_u32(uint32_t *a, uint32_t *b, uint32_t n, uint32_t root, uint32_t mod) {
    int rc = orc_ntt_u32(a, n, root, mod, -1);
    if (!rc)
        rc = orc_ntt_u32(b, n, root, mod, -1);
    if (rc)
        return rc;
    for (uint32_t i = 0; i < n; ++i)
        a[i] = (uint32_t)((uint64_t)a[i] * b[i] % mod);
    return orc_intt_u32(a, n, root, mod);
}

int orc_cyclic_conv_gl64(uint64_t *a, uint64_t *b, uint32_t n) {
    int lg = log2_exact(n);
    if (lg < 0)
        return -1;
    const uint64_t root = orc_gl_root((uint32_t)lg);
    int rc = orc_ntt_gl64(a, n, root, -1);
    if (!rc)
        rc = orc_ntt_gl64(b, n, root, -1);
    if (rc)
        return rc;
    for (uint32_t i = 0; i < n; ++i)
        a[i] = orc_gl_mul(a[i], b[i]);
    return orc_intt_gl64(a, n, root);
}

uint64_t orc_fnv1a64(const void *data, size_t nbytes) {
    const unsigned char *p = (const unsigned char *)data;
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < nbytes; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}
