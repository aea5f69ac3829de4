// api.cu -- host side of libstntt: parameters, plans, twiddle cache,
// workspaces and the C ABI declared in include/stntt.h.
//
// Reference boundary this replaces: cuda::ntt::NttArgs / getNttKernelArgs /
// autoNtt<n> (src/cuda/ntt/ntt_kernel.cuh:31-200), which allocate, upload a
// freshly built twiddle table (initTwiddles, .../implementations/common.cuh:
// 17-109) and launch on every call, and exit the process on CUDA errors
// (CCErr, src/cuda/cu_util.cuh:12-28). Here a context caches device-built
// twiddle tables and plans, runs asynchronously on the caller's stream and
// returns a status.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/stntt.h"
#include "internal.h"
#include "ctx_internal.h"

namespace stntt {

cudaError_t launch_tile_u32(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t, cudaStream_t,
                             const void *, int *);
cudaError_t launch_tile_u32l(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t, cudaStream_t,
                             const void *, int *);
cudaError_t batch_prepare_u32l(size_t, int *);
cudaError_t batch_launch_u32l(const void *, const void *, unsigned long long, unsigned int *, void *, size_t, unsigned,
                              unsigned, cudaStream_t);
cudaError_t launch_tile_gl64(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t, cudaStream_t,
                             const void *, int *);
cudaError_t gen_powers_u32(void *, uint64_t, uint64_t, uint64_t, uint32_t, cudaStream_t);
cudaError_t gen_four_step_u32(void *, const void *, const void *, uint32_t, uint32_t, uint64_t, uint32_t,
                               cudaStream_t);
cudaError_t gen_four_step_gl64(void *, const void *, const void *, uint32_t, uint32_t, uint64_t, uint32_t,
                                cudaStream_t);
cudaError_t gen_powers_gl64(void *, uint64_t, uint64_t, uint64_t, cudaStream_t);
cudaError_t pointwise_u32(const void *, const void *, void *, size_t, uint32_t, cudaStream_t);
cudaError_t pointwise_gl64(const void *, const void *, void *, size_t, cudaStream_t);
cudaError_t fill_uniform_u32(void *, size_t, uint64_t, uint32_t, cudaStream_t);
cudaError_t fill_uniform_gl64(void *, size_t, uint64_t, cudaStream_t);
cudaError_t copy_scale_u32(const void *, void *, size_t, uint64_t, uint32_t, cudaStream_t);
cudaError_t copy_scale_gl64(const void *, void *, size_t, uint64_t, cudaStream_t);
cudaError_t launch_gl_probe(uint64_t *, unsigned, int, cudaStream_t);
cudaError_t launch_find_params(uint64_t, uint64_t, uint64_t *, cudaStream_t);
cudaError_t preload_u32();
cudaError_t launch_cluster_u32l(const PassDesc &, const PassDesc &, uint32_t, const void *, const void *, void *,
                                uint64_t, uint32_t, uint32_t, size_t, uint32_t, cudaStream_t);
cudaError_t launch_cluster_gl64(const PassDesc &, const PassDesc &, uint32_t, const void *, const void *, void *,
                                uint64_t, uint32_t, uint32_t, size_t, uint32_t, cudaStream_t);
cudaError_t preload_u32l();
cudaError_t preload_gl64();
cudaError_t preload_tma_u32l();
cudaError_t preload_tma_gl64();
size_t batch_args_size_u32();
size_t batch_args_size_gl64();
void batch_args_fill_u32(const PassDesc &, uint32_t, const void *, const unsigned long long *,
                         const unsigned long long *, uint64_t, void *);
void batch_args_fill_gl64(const PassDesc &, uint32_t, const void *, const unsigned long long *,
                          const unsigned long long *, uint64_t, void *);
cudaError_t batch_prepare_u32(size_t, int *);
cudaError_t batch_prepare_gl64(size_t, int *);
cudaError_t batch_launch_u32(const void *, const void *, unsigned long long, unsigned int *, void *, size_t, unsigned,
                             unsigned, cudaStream_t);
cudaError_t batch_launch_gl64(const void *, const void *, unsigned long long, unsigned int *, void *, size_t,
                              unsigned, unsigned, cudaStream_t);

static constexpr uint64_t GL_P = 0xFFFFFFFF00000001ull;
typedef unsigned __int128 u128;

uint64_t host_pow_mod(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1)
            r = (uint64_t)((u128)r * b % m);
        b = (uint64_t)((u128)b * b % m);
        e >>= 1;
    }
    return r;
}
uint64_t host_gl_mul(uint64_t a, uint64_t b) { return (uint64_t)((u128)a * b % GL_P); }
uint64_t host_gl_pow(uint64_t b, uint64_t e) { return host_pow_mod(b, e, GL_P); }
uint64_t host_tw_entry(int field, uint64_t w, uint32_t p) {
    if (field == kFieldGL)
        return w;
    const uint64_t wp = (w << 32) / p;  // Shoup companion floor(w * 2^32 / p)
    return (w & 0xffffffffull) | (wp << 32);
}

cudaError_t launch_tile_vec_gl64f(const PassDesc &, const void *, const void *, void *, uint64_t, cudaStream_t);
cudaError_t launch_tile_vec_gl64i(const PassDesc &, const void *, const void *, void *, uint64_t, cudaStream_t);
cudaError_t launch_tile_vec_u32l(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t,
                                 cudaStream_t);
cudaError_t preload_vec_gl64f();
cudaError_t preload_vec_gl64i();
cudaError_t preload_vec_u32l();

cudaError_t launch_tile_vc_gl64(const PassDesc &, const void *, const void *, void *, uint64_t, cudaStream_t);
cudaError_t launch_tile_vc_u32l(const PassDesc &, uint32_t, const void *, const void *, void *, uint64_t,
                                cudaStream_t);
cudaError_t preload_vc_gl64();
cudaError_t preload_vc_u32l();

cudaError_t launch_tile_vc(int field, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                           uint64_t batch, cudaStream_t s) {
    if (field == kFieldGL)
        return launch_tile_vc_gl64(d, tables, in, out, batch, s);
    if (p < (1u << 30))
        return launch_tile_vc_u32l(d, p, tables, in, out, batch, s);
    return cudaErrorNotSupported;
}

cudaError_t preload_vc() {
    const cudaError_t e = preload_vc_gl64();
    return e == cudaSuccess ? preload_vc_u32l() : e;
}

cudaError_t launch_tile_vec(int field, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                            uint64_t batch, cudaStream_t s) {
    if (d.vcl)
        return launch_tile_vc(field, d, p, tables, in, out, batch, s);
    if (field == kFieldGL)  // built for the two standard roots only (see PassDesc::pow2)
        return d.pow2 == 1   ? launch_tile_vec_gl64f(d, tables, in, out, batch, s)
               : d.pow2 == 2 ? launch_tile_vec_gl64i(d, tables, in, out, batch, s)
                             : cudaErrorNotSupported;
    // the lazy 32-bit field with bound-tracked DFTs, which need 8p < 2^32
    // (every findParams prime up to n = 2^26); other primes take the plain tile
    if (p < (1u << 29))
        return launch_tile_vec_u32l(d, p, tables, in, out, batch, s);
    return cudaErrorNotSupported;
}

cudaError_t preload_vec() {
    cudaError_t e = preload_vec_gl64f();
    if (e == cudaSuccess)
        e = preload_vec_gl64i();
    if (e == cudaSuccess)
        e = preload_vc();
    return e == cudaSuccess ? preload_vec_u32l() : e;
}

cudaError_t preload_kernels() {
    cudaError_t e = preload_u32();
    if (e == cudaSuccess)
        e = preload_u32l();
    if (e == cudaSuccess)
        e = preload_gl64();
    if (e == cudaSuccess)
        e = preload_tma_u32l();
    if (e == cudaSuccess)
        e = preload_tma_gl64();
    if (e == cudaSuccess)
        e = preload_vec();
    return e;
}

cudaError_t launch_tile(int field, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                        uint64_t batch, cudaStream_t s, const void *in2, int *err) {
    if (d.vec && !in2) {  // the vector-lines build where the pass and its pointers allow it
        const cudaError_t e = launch_tile_vec(field, d, p, tables, in, out, batch, s);
        if (e != cudaErrorNotSupported)
            return e;
    }
    if (field == kFieldGL)
        return launch_tile_gl64(d, p, tables, in, out, batch, s, in2, err);
    // lazy reduction needs 4p < 2^32
    return p < (1u << 30) ? launch_tile_u32l(d, p, tables, in, out, batch, s, in2, err)
                          : launch_tile_u32(d, p, tables, in, out, batch, s, in2, err);
}
cudaError_t launch_gen_powers(int field, void *out, uint64_t count, uint64_t base, uint64_t scale, uint32_t p,
                              cudaStream_t s) {
    return field == kFieldGL ? gen_powers_gl64(out, count, base, scale, s)
                             : gen_powers_u32(out, count, base, scale, p, s);
}
cudaError_t launch_cluster(int field, const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                           const void *in, void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem,
                           uint32_t log_k, cudaStream_t s) {
    if (field == kFieldGL)
        return launch_cluster_gl64(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
    if (p < (1u << 30))
        return launch_cluster_u32l(d1, d2, p, tables, in, out, batch, xoff, xs, smem, log_k, s);
    return cudaErrorNotSupported;
}
cudaError_t gen_four_step_mont_u32(void *, const void *, const void *, uint32_t, uint32_t, uint64_t, uint32_t,
                                   cudaStream_t);
cudaError_t launch_gen_four_step_mont(void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS,
                                      uint64_t count, uint32_t p, cudaStream_t s) {
    return gen_four_step_mont_u32(out, lo, hi, h, logS, count, p, s);
}
cudaError_t launch_gen_four_step(int field, void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS,
                                 uint64_t count, uint32_t p, cudaStream_t s) {
    return field == kFieldGL ? gen_four_step_gl64(out, lo, hi, h, logS, count, p, s)
                             : gen_four_step_u32(out, lo, hi, h, logS, count, p, s);
}
cudaError_t launch_pointwise(int field, const void *a, const void *b, void *out, size_t count, uint32_t p,
                             cudaStream_t s) {
    return field == kFieldGL ? pointwise_gl64(a, b, out, count, s) : pointwise_u32(a, b, out, count, p, s);
}
cudaError_t launch_fill_uniform(int field, void *out, size_t count, uint64_t seed, uint32_t p, cudaStream_t s) {
    return field == kFieldGL ? fill_uniform_gl64(out, count, seed, s) : fill_uniform_u32(out, count, seed, p, s);
}
cudaError_t launch_copy_scale(int field, const void *in, void *out, size_t count, uint64_t scale_tw, uint32_t p,
                              cudaStream_t s) {
    return field == kFieldGL ? copy_scale_gl64(in, out, count, scale_tw, s)
                             : copy_scale_u32(in, out, count, scale_tw, p, s);
}

// ---------------------------------------------------------------------------
// findParams (src/ntt/ntt_util.cpp:10-49): smallest prime mod = k*size + 1
// >= min_mod (trial division), smallest generator g, root = g^((mod-1)/size).
// ---------------------------------------------------------------------------
static uint64_t isqrt_u64(uint64_t n) {
    uint64_t r = 0;
    for (uint64_t bit = 1ull << 31; bit; bit >>= 1) {
        const uint64_t c = r | bit;
        if (c <= n / c)
            r = c;
    }
    return r;
}
static bool is_prime_td(uint64_t n) {
    if (n < 2)
        return n == 1;  // the reference's isPrime(1) is vacuously true; never reached (mod >= 2)
    const uint64_t e = isqrt_u64(n);
    for (uint64_t x = 2; x <= e; ++x)
        if (n % x == 0)
            return false;
    return true;
}
static std::vector<uint64_t> prime_factors(uint64_t n) {
    std::vector<uint64_t> f;
    for (uint64_t i = 2; i <= isqrt_u64(n); ++i) {
        if (n % i == 0) {
            f.push_back(i);
            while (n % i == 0)
                n /= i;
        }
    }
    if (n > 1)
        f.push_back(n);
    return f;
}

}  // namespace stntt

using namespace stntt;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
namespace sd {

// Elements per work item of the persistent batched launch (C columns or rows
// of L points, 16 per thread, 512 threads).
constexpr uint32_t kBatchTileLog = 13;

struct PlanKey {
    int field;
    uint32_t log_n, p;
    uint64_t root;  // root of the direction (inverse: root^-1)
    int dir;
    int kind;         // the shape set it was built from: kPlanAll, kPlanSmall or kPlanBatched
    bool small_call;  // for calls of fewer than kSmallCallElems elements (smaller full twiddle tables)
    bool operator<(const PlanKey &o) const {
        return std::tie(field, log_n, p, root, dir, kind, small_call) <
               std::tie(o.field, o.log_n, o.p, o.root, o.dir, o.kind, o.small_call);
    }
};

struct Plan {
    int field = 0;
    uint32_t log_n = 0, p = 0;
    std::vector<PassDesc> passes;
    void *d_tables = nullptr;
    size_t table_bytes = 0;
};

struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// A stream's scratch buffer and when it was last handed out.
struct StreamBuf {
    DevBuf buf;
    uint64_t last_use = 0;
};

// Streams whose scratch a context keeps at once (the serving loop uses one
// per slot, up to 32); beyond this the least recently used buffer is freed.
constexpr size_t kMaxStreamWorkspaces = 64;
// Bytes after each stream's scratch, zeroed when it is allocated: the grid
// barrier of the one-launch two-pass kernel (coop.cuh).
constexpr size_t kWorkspaceTail = 256;

// A plan shape chosen by the caller (the autotuner) instead of the default.
struct PlanSpec {
    std::vector<uint32_t> logs, elems, cols;
};

}  // namespace sd
using namespace sd;

struct stntt_ctx {
    int device = 0;
    std::mutex mu;
    std::map<PlanKey, std::unique_ptr<Plan>> plans;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t, int>, DevBuf> stage_tables;  // (log_n, p, root, wrap)
    std::map<cudaStream_t, StreamBuf> workspaces;
    uint64_t ws_clock = 0;
    std::map<std::tuple<int, uint32_t, int>, PlanSpec> specs;  // (field, log_n, kind) -> override
    cudaStream_t setup = nullptr;
    // host-buffer calls: one at a time, on their own stream and staging buffer
    std::mutex host_mu;
    cudaStream_t host_stream = nullptr;
    DevBuf host_stage;
    // CUDA events around the device work of the last host-buffer call, and
    // its duration (the reference's autoNtt returns this "kernel time")
    cudaEvent_t host_ev0 = nullptr, host_ev1 = nullptr;
    float host_kernel_ms = 0.f;
    std::string err;
    size_t mem = 0;
    uint32_t cluster_log = 3;  // log2 of the cluster size the one-launch transforms use (3 or 4)
    int tma_mode = -1;         // TMA-staged passes: -1 built-in choice, 0 never, 1 wherever a pass allows
    int coop_mode = 0;         // one cooperative launch for small two-pass calls: 1 where it fits, 0 never
    int *d_err = nullptr;      // device error word of the staged kernels' bounded waits
};

namespace sd {

int fail(stntt_ctx *ctx, int status, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->mu);
        ctx->err = msg;
    }
    return status;
}
int cuda_fail(stntt_ctx *ctx, cudaError_t e, const char *what) {
    return fail(ctx, STNTT_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess)
            prev = -1;
        if (prev != dev)
            err = cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

uint32_t ilog2(uint64_t v) {
    uint32_t l = 0;
    while ((1ull << l) < v)
        ++l;
    return l;
}

// Field root of order 2^log_n for the given direction.
uint64_t dir_root(int field, uint64_t root, uint32_t p, int dir) {
    if (dir == STNTT_FORWARD)
        return root;
    return field == kFieldGL ? host_gl_pow(root, GL_P - 2) : host_pow_mod(root, p - 2, p);
}
uint64_t fpow(int field, uint64_t b, uint64_t e, uint32_t p) {
    return field == kFieldGL ? host_gl_pow(b, e) : host_pow_mod(b, e, p);
}
uint64_t fmul(int field, uint64_t a, uint64_t b, uint32_t p) {
    return field == kFieldGL ? host_gl_mul(a, b) : (uint64_t)((u128)a * b % p);
}

// Shared-memory stride between a CTA's columns (elements): the padded length
// rounded up to a residue, modulo the bank count (16 eight-byte or 32
// four-byte banks), that spreads one warp access over the banks. Threads
// running along a column (tfast): U threads per column, residue U. Threads
// across columns: C columns side by side, residue banks / C; from C = banks
// up every thread of a phase reads the same row of C different columns, so
// the residue must be odd. (A simulation of every step's accesses chose these;
// an even stride there made all C columns hit one bank.)
uint32_t column_stride(int field, uint32_t L, uint32_t C, uint32_t U, uint32_t tfast) {
    const uint32_t padshift = field == kFieldGL ? 4 : 5;
    const uint32_t banks = field == kFieldGL ? 16 : 32;
    const uint32_t base = L + (L >> padshift);
    uint32_t want;
    if (tfast)
        want = U < banks ? U : 0;
    else
        want = C < banks ? banks / C : 1;
    return base + ((want + banks - base % banks) % banks);
}

// Tile geometry for one pass: elements per thread E, columns per CTA C,
// shared-memory column stride and size.
void shape_pass(PassDesc &d, int field, uint64_t col_limit, uint32_t want_E, uint32_t want_C) {
    const uint32_t L = 1u << d.logL;
    // Defaults from the autotuner's sweeps on GB300 (both fields, 2^16..2^26):
    // 16 elements per thread, C = min(8, 8192 / L) columns per CTA for 8-byte
    // values and min(16, 8192 / L) for 4-byte ones (64-byte row segments).
    d.E = L < 16 ? L : 16;
    if (L >= 16 && (want_E == 16 || want_E == 32) && want_E <= L)
        d.E = want_E;
    if (want_E == 8 && d.logL >= 7 && d.logL <= 11)  // the 8-element compile-time builds
        d.E = 8;
    const uint32_t U = L / d.E;
    const uint32_t max_threads = d.E >= 32 ? 512 : 1024;
    uint64_t C;
    if (want_C) {
        C = want_C;
    } else if (d.mode == kModeRow && d.logN == d.logL) {
        C = std::max<uint64_t>(1, 256 / U);  // whole transforms per CTA: ~256 threads
    } else {
        C = std::min<uint64_t>(field == kFieldGL ? 8 : 16, 8192 / L);
    }
    C = std::min<uint64_t>(C, max_threads / U);
    C = std::min<uint64_t>(C, col_limit);
    C = std::min<uint64_t>(C, 64);
    C = std::max<uint64_t>(C, 1);
    const size_t esz = field == kFieldGL ? 8 : 4;
    while (C > 1 && C * (L + (L >> 4) + 32) * esz > 200 * 1024)  // shared-memory budget per CTA
        C >>= 1;
    d.logC = ilog2(C);
    d.threads = (uint32_t)(C * U);
    d.cs = column_stride(field, L, (uint32_t)C, U, d.tfast);
    d.smem_bytes = (size_t)C * d.cs * (field == kFieldGL ? 8 : 4);
}

// The vector-lines build of a pass (tile_v.cuh), when asked for (STNTT_PASS_VEC
// in a plan's elements per thread) and the pass allows it: a pass of a
// multi-pass plan, E = 16 (or 8) points per line per thread, V = 16 bytes / w
// lines per thread and C = V * 2^g lines per CTA, C dividing the pass's lines
// per sub-problem. Tiles of 2^7..2^10 points take g = 3 or 2 (within 1024
// threads), the wide tiles of two-pass plans (2^11 and 2^12 points) g = 2 or
// 1 within 512 threads; 200 KiB of shared memory at most. want_C picks C (0:
// the most line groups that fit).
size_t vec_smem(uint32_t V, uint32_t logG, uint32_t logL, uint32_t w) {
    const uint32_t pb = logG < 2 ? 3 - logG : 0;  // one 16-byte pad per 2^pb points (tile_v.cuh, vpoint)
    return ((size_t)V << logG) * (1u << logL) * w + (pb ? (size_t)((1u << logL) >> pb) * 16 : 0);
}

void shape_pass_vec(PassDesc &d, int field, uint64_t col_limit, uint32_t want_E, uint32_t want_C) {
    d.vec = 0;
    if (d.logL < 7 || d.logL > 12 || d.do_scale || d.logL >= d.logN)
        return;
    const uint32_t V = field == kFieldGL ? 2 : 4, w = field == kFieldGL ? 8 : 4;
    d.vE = (want_E == 4 || want_E == 8) ? want_E : 16;
    if (d.vE == 4 && (d.logL < 9 || d.logL > 11))  // 4 points per line: built for 2^9..2^11-point passes
        return;
    const uint32_t U = (1u << d.logL) / d.vE;
    const uint32_t gmax = d.logL <= 10 ? 3 : 2, gmin = d.logL <= 10 ? 2 : 0;
    const uint32_t tmax = d.logL <= 10 ? 1024 : 512;
    uint32_t logG = gmax;
    for (uint32_t g = gmin; g <= gmax; ++g)
        if (want_C == (V << g))
            logG = g;
    while (logG > gmin && (((uint64_t)V << logG) > col_limit || vec_smem(V, logG, d.logL, w) > 200 * 1024 ||
                           (U << logG) > tmax))
        --logG;
    if (((uint64_t)V << logG) > col_limit || (U << logG) > tmax || vec_smem(V, logG, d.logL, w) > 200 * 1024)
        return;
    d.vec = V;
    d.vlogG = logG;
    d.vthreads = U << logG;
    d.vsmem = vec_smem(V, logG, d.logL, w);
}

// The vector-lines cluster build of a pass (tile_vc.cuh), when asked for
// (STNTT_PASS_CLUSTER with STNTT_PASS_VEC): passes of 2^11..2^13 points, 8
// points per line, clusters of 8 CTAs, the first phase over 2^ceil(logL/2)
// points; C = V * 4 or V * 8 lines per cluster, one CTA's threads within 1024
// and its registers (64 or 80 per thread) within the SM's 65536.
void shape_pass_vc(PassDesc &d, int field, uint64_t col_limit, uint32_t want_C) {
    d.vcl = 0;
    if (d.logL < 11 || d.logL > 13 || d.do_scale || d.logL >= d.logN)
        return;
    const uint32_t V = field == kFieldGL ? 2 : 4, w = field == kFieldGL ? 8 : 4, regs = field == kFieldGL ? 80 : 64;
    const uint32_t logK = 3, log1 = (d.logL + 1) / 2;
    uint32_t logG = want_C == (V << 2) ? 2 : 3;
    const auto threads = [&](uint32_t g) { return (1u << (d.logL - log1 - logK + g)) * ((1u << log1) / 8); };
    const auto smem = [&](uint32_t g) { return ((size_t)V << g) * (1u << d.logL) * w >> logK; };
    while (logG > 2 && (((uint64_t)V << logG) > col_limit || threads(logG) > 1024 || threads(logG) * regs > 65536 ||
                        smem(logG) > 200 * 1024))
        --logG;
    if (((uint64_t)V << logG) > col_limit || threads(logG) > 1024 || threads(logG) * regs > 65536 ||
        smem(logG) > 200 * 1024)
        return;
    d.vec = V;
    d.vE = 8;
    d.vlogG = logG;
    d.vcl = logK;
    d.vlog1 = log1;
    d.vthreads = threads(logG);
    d.vsmem = smem(logG);
}

// Whether a pass runs TMA-staged (tma.cuh) by default; the kernel still
// falls back to the plain one where the pass does not allow it.
uint32_t tma_builtin(int field, const PassDesc &d) {
    (void)field;
    (void)d;
    return 0;
}

// Largest column-pass sub-problem (log2 points) of a pass of a call of 2^22+
// elements that reads its four-step twiddle from a full table, for the plain
// build (kFullTwiddleMaxLog, or STNTT_FULL_TWIDDLE_MAX_LOG from the
// environment) and the vector-lines build (kFullTwiddleMaxLogVec, or
// STNTT_FULL_TWIDDLE_MAX_LOG_VEC); 14..26, read once.
uint32_t env_log_limit(const char *name, uint32_t dflt) {
    const char *e = getenv(name);
    const long x = e ? strtol(e, nullptr, 10) : -1;
    return (x >= (long)kFullTwiddleMinLog && x <= 26) ? (uint32_t)x : dflt;
}
uint32_t full_twiddle_max_log(bool vec) {
    static const uint32_t plain = env_log_limit("STNTT_FULL_TWIDDLE_MAX_LOG", kFullTwiddleMaxLog);
    static const uint32_t v = env_log_limit("STNTT_FULL_TWIDDLE_MAX_LOG_VEC", kFullTwiddleMaxLogVec);
    return vec ? v : plain;
}
// The same for calls of fewer than 2^22 elements: kFullTwiddleMaxLogSmall
// (plain build) and kFullTwiddleMaxLogSmallVec (vector-lines build), or
// STNTT_FULL_TWIDDLE_MAX_LOG_SMALL for both.
uint32_t full_twiddle_max_log_small(bool vec) {
    static const uint32_t plain = env_log_limit("STNTT_FULL_TWIDDLE_MAX_LOG_SMALL", kFullTwiddleMaxLogSmall);
    static const uint32_t v = env_log_limit("STNTT_FULL_TWIDDLE_MAX_LOG_SMALL", kFullTwiddleMaxLogSmallVec);
    return vec ? v : plain;
}

// Smallest column-pass sub-problem (log2 points) whose full four-step table
// holds 4-byte Montgomery entries in the 32-bit vector-lines build, for calls
// of 2^22+ elements: 2^17 (kFullMontMinLog), or STNTT_FULL_MONT_MIN_LOG
// (14..26) from the environment, read once. Half the bytes of a Shoup pair
// per element for one more multiply: the 2^17-point table of the second pass
// of a 2^26-point transform stays in L2 either way, but its 8-byte loads kept
// the L1 data pipe busy (measured forward + inverse 0.808 -> 0.800 ms).
// Small calls and batched plans keep Shoup pairs up to 2^20 points (the
// batched items read Shoup tables only).
uint32_t full_mont_min_log(bool small_or_batched) {
    static const uint32_t v = env_log_limit("STNTT_FULL_MONT_MIN_LOG", kFullMontMinLog);
    return small_or_batched ? kFullTwiddleMaxLog + 1 : v;
}

// -p^-1 mod 2^32 for odd p (Newton's iteration doubles the correct low bits).
uint32_t neg_inv32(uint32_t p) {
    uint32_t x = p;  // p * p = 1 mod 8: three bits
    for (int i = 0; i < 4; ++i)
        x *= 2u - p * x;
    return 0u - x;
}

// Build the pass list and the twiddle tables for one transform.
int build_plan(stntt_ctx *ctx, Plan &pl, int field, uint32_t log_n, uint32_t p, uint64_t root_dir, int dir,
               const PlanSpec *spec, bool small_call, bool batched) {
    pl.field = field;
    pl.log_n = log_n;
    pl.p = p;
    if (log_n == 0)
        return STNTT_OK;
    const uint64_t n = 1ull << log_n;
    const uint32_t single_max = 13, tile_max = 12;
    std::vector<uint32_t> logs;
    if (spec) {
        logs = spec->logs;
    } else if (log_n <= single_max) {
        logs.push_back(log_n);
    } else {
        const uint32_t K = (log_n + tile_max - 1) / tile_max;
        for (uint32_t i = 0; i < K; ++i)
            logs.push_back(log_n / K + (i < log_n % K ? 1 : 0));
    }
    const uint32_t K = (uint32_t)logs.size();
    // Tables, generated in this order into one allocation: powers (count,
    // base, scale), or a column pass's full four-step table (built from its
    // lo / hi tables, which come earlier).
    struct TableReq {
        uint64_t at, count, base, scale;
        bool full;
        uint64_t lo_off, hi_off;
        uint32_t h, logS;
        bool mont;  // full table of 4-byte Montgomery entries (count = entries)
    };
    std::vector<TableReq> reqs;
    uint64_t off = 0;
    // every table starts on a 32-byte boundary (vector loads of 2 or 4 entries)
    auto add_table = [&](uint64_t count, uint64_t base, uint64_t scale) {
        off = (off + 3) & ~3ull;
        reqs.push_back({off, count, base, scale, false, 0, 0, 0, 0, false});
        const uint64_t o = off;
        off += count;
        return o;
    };
    auto add_full = [&](uint64_t count, uint64_t lo_off, uint64_t hi_off, uint32_t h, uint32_t logS, bool mont) {
        off = (off + 3) & ~3ull;
        reqs.push_back({off, count, 0, 0, true, lo_off, hi_off, h, logS, mont});
        const uint64_t o = off;
        off += mont ? (count + 1) / 2 : count;  // 4-byte Montgomery entries take half the 8-byte slots
        return o;
    };
    const uint64_t modulus = field == kFieldGL ? GL_P : p;
    const uint64_t ninv = dir == STNTT_INVERSE ? fpow(field, n % modulus, modulus - 2, p) : 1;  // n^-1
    uint32_t done = 0;  // log2 of the product of the lengths of earlier passes
    for (uint32_t i = 0; i < K; ++i) {
        PassDesc d;
        d.logL = logs[i];
        d.logN = log_n;
        const uint32_t L = 1u << d.logL;
        const uint64_t wL = fpow(field, root_dir, n >> d.logL, p);  // w_L = w_n^(n/L)
        d.tw_off = add_table(L, wL, 1);
        // radix-16 internal roots (for L < 16: entry j*16/L = w_L^j)
        if (L >= 16) {
            const uint64_t w16 = fpow(field, wL, L / 16, p);
            for (int j = 0; j < 8; ++j)
                d.wR[j] = host_tw_entry(field, fpow(field, w16, j, p), p);
        } else {
            for (uint32_t j = 0; j < L / 2; ++j)
                d.wR[j * 16 / L] = host_tw_entry(field, fpow(field, wL, j, p), p);
        }
        if (field == kFieldGL) {  // the standard roots 7^((p-1)/n) and their inverses: w_16 = 2^156 / 2^36
            const uint64_t fwd = host_gl_pow(7, (GL_P - 1) >> log_n);
            d.pow2 = root_dir == fwd ? 1 : root_dir == host_gl_pow(fwd, GL_P - 2) ? 2 : 0;
        }
        d.scale = host_tw_entry(field, ninv, p);
        uint64_t col_limit;
        if (i + 1 < K) {
            d.mode = kModeCol;
            d.tfast = 0;
            d.logM = log_n - done;
            d.logS = d.logM - d.logL;
            d.h = (d.logM + 1) / 2;
            const uint64_t wM = fpow(field, root_dir, n >> d.logM, p);
            d.lo_off = add_table(1ull << d.h, wM, 1);
            d.hi_off = add_table(1ull << (d.logM - d.h), fpow(field, wM, 1ull << d.h, p), i == 0 ? ninv : 1);
            col_limit = 1ull << d.logS;
        } else {
            d.mode = kModeRow;
            d.tfast = (K == 1) ? 1 : 0;
            d.do_scale = (K == 1 && dir == STNTT_INVERSE) ? 1 : 0;
            d.logN1 = K >= 2 ? logs[0] : 0;
            d.logN2 = K == 3 ? logs[1] : 0;
            col_limit = 1ull << 20;
        }
        const uint32_t want_e = spec ? spec->elems[i] : 0;
        shape_pass(d, field, col_limit, want_e & 0xffu, (want_e & STNTT_PASS_VEC) ? 0 : (spec ? spec->cols[i] : 0));
        if (K > 1 && (want_e & STNTT_PASS_VEC)) {
            if (d.mode == kModeRow)
                col_limit = std::min<uint64_t>(col_limit, 1ull << (log_n - d.logL));
            shape_pass_vec(d, field, col_limit, want_e & 0xffu, spec ? spec->cols[i] : 0);
            if (want_e & STNTT_PASS_CLUSTER)
                shape_pass_vc(d, field, col_limit, spec ? spec->cols[i] : 0);
        }
        // Column passes over 2^14..2^20-point sub-problems read the twiddle
        // w_M^(col*pos) from a table laid out like the data: one load and one
        // product per element instead of two lookups and two products (M
        // entries per plan; the lo / hi tables stay for the kernels without
        // this path). Passes in the vector-lines build, whose table loads are
        // 16 bytes wide, use it up to 2^26-point sub-problems: the table then
        // streams from HBM beside the data and still wins (measured on GB300,
        // forward + inverse: Goldilocks 2^24 0.669 -> 0.631 ms, 2^22 0.186 ->
        // 0.176 ms, 32-bit 2^26 1.015 -> 0.994 ms), at n * 8 bytes of table per
        // plan. STNTT_FULL_TWIDDLE_MAX_LOG and STNTT_FULL_TWIDDLE_MAX_LOG_VEC
        // (14..26) move the limits of calls of 2^22+ elements.
        if (d.mode == kModeCol && d.logM >= kFullTwiddleMinLog &&
            d.logM <= (small_call ? full_twiddle_max_log_small(d.vec != 0) : full_twiddle_max_log(d.vec != 0))) {
            // Beyond 2^20 points the 32-bit table streams from HBM: there its
            // entries are 4-byte Montgomery values instead of 8-byte Shoup
            // pairs (a 2^26-point table: 256 MiB instead of 512 MiB to read
            // beside the 256 MiB of data), at two more multiplies per product.
            d.full_mont =
                (field != kFieldGL && d.vec && d.logM >= full_mont_min_log(small_call || batched) && p < (1u << 29))
                    ? 1
                    : 0;
            d.pinv = d.full_mont ? neg_inv32(p) : 0;
            d.full_off = add_full(1ull << d.logM, d.lo_off, d.hi_off, d.h, d.logS, d.full_mont != 0);
        }
        d.tma = ctx->tma_mode < 0 ? tma_builtin(field, d) : (uint32_t)ctx->tma_mode;
        pl.passes.push_back(d);
        done += d.logL;
    }
    const size_t esz = 8;  // both fields: 8-byte twiddle entries
    pl.table_bytes = off * esz;
    cudaError_t e = cudaMalloc(&pl.d_tables, pl.table_bytes);
    if (e != cudaSuccess) {
        pl.d_tables = nullptr;
        return cuda_fail(ctx, e, "cudaMalloc(twiddle tables)");
    }
    char *tb = static_cast<char *>(pl.d_tables);
    for (const auto &r : reqs) {
        e = r.mont   ? launch_gen_four_step_mont(tb + r.at * esz, tb + r.lo_off * esz, tb + r.hi_off * esz, r.h, r.logS,
                                                 r.count, p, ctx->setup)
            : r.full ? launch_gen_four_step(field, tb + r.at * esz, tb + r.lo_off * esz, tb + r.hi_off * esz, r.h,
                                            r.logS, r.count, p, ctx->setup)
                     : launch_gen_powers(field, tb + r.at * esz, r.count, r.base, r.scale, p, ctx->setup);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "twiddle generation launch");
    }
    e = cudaStreamSynchronize(ctx->setup);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "twiddle generation");
    return STNTT_OK;
}

int get_plan(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t p, uint64_t root, int dir, const Plan **out,
             int kind) {
    const uint64_t rd = dir_root(field, root, p, dir);
    std::lock_guard<std::mutex> g(ctx->mu);
    // a small call (batched launch) uses the small-call (batched) shape when
    // one is set, else the plan of every call
    const bool small_call = kind == kPlanSmall;
    if (kind != kPlanAll && !ctx->specs.count({field, log_n, kind}))
        kind = kPlanAll;
    PlanKey key{field, log_n, field == kFieldGL ? 0u : p, rd, dir, kind, small_call};
    auto it = ctx->plans.find(key);
    if (it != ctx->plans.end()) {
        *out = it->second.get();
        return STNTT_OK;
    }
    auto pl = std::make_unique<Plan>();
    PlanSpec spec;
    auto sit = ctx->specs.find({field, log_n, kind});
    const bool has_spec = sit != ctx->specs.end();
    if (has_spec)
        spec = sit->second;
    ctx->mu.unlock();
    int rc = build_plan(ctx, *pl, field, log_n, p, rd, dir, has_spec ? &spec : nullptr, small_call,
                        kind == kPlanBatched);
    ctx->mu.lock();
    if (rc != STNTT_OK) {
        if (pl->d_tables)
            cudaFree(pl->d_tables);
        return rc;
    }
    void *mine = pl->d_tables;
    auto ins = ctx->plans.emplace(key, std::move(pl));
    if (ins.second)
        ctx->mem += ins.first->second->table_bytes;
    else if (mine)
        cudaFree(mine);  // another thread built the same plan first
    *out = ins.first->second.get();
    return STNTT_OK;
}

// Per-stream scratch of at least `bytes`. A buffer that must grow, and the
// least recently used one when a stream beyond kMaxStreamWorkspaces appears,
// is taken out of the map under the lock and waited for and freed outside it,
// so other threads on the context do not stall behind that wait.
int get_workspace(stntt_ctx *ctx, cudaStream_t s, size_t bytes, void **ptr, void **tail) {
    StreamBuf old, victim;
    cudaStream_t victim_s = nullptr;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        auto it = ctx->workspaces.find(s);
        if (it != ctx->workspaces.end() && it->second.buf.bytes >= bytes) {
            it->second.last_use = ++ctx->ws_clock;
            *ptr = it->second.buf.ptr;
            if (tail)
                *tail = static_cast<char *>(it->second.buf.ptr) + it->second.buf.bytes;
            return STNTT_OK;
        }
        if (it != ctx->workspaces.end()) {
            old = it->second;
            ctx->workspaces.erase(it);
        } else if (ctx->workspaces.size() >= kMaxStreamWorkspaces) {
            auto lru = ctx->workspaces.begin();
            for (auto j = ctx->workspaces.begin(); j != ctx->workspaces.end(); ++j)
                if (j->second.last_use < lru->second.last_use)
                    lru = j;
            victim = lru->second;
            victim_s = lru->first;
            ctx->workspaces.erase(lru);
        }
        ctx->mem -= (old.buf.ptr ? old.buf.bytes + kWorkspaceTail : 0) +
                    (victim.buf.ptr ? victim.buf.bytes + kWorkspaceTail : 0);
    }
    if (old.buf.ptr) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "workspace resize: waiting for the stream");
        cudaFree(old.buf.ptr);
    }
    if (victim.buf.ptr) {
        if (cudaStreamSynchronize(victim_s) != cudaSuccess) {  // e.g. a stream destroyed without release
            cudaGetLastError();
            cudaDeviceSynchronize();
        }
        cudaFree(victim.buf.ptr);
    }
    StreamBuf nb;
    bytes = (bytes + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&nb.buf.ptr, bytes + kWorkspaceTail);
    if (e != cudaSuccess)
        return fail(ctx, e == cudaErrorMemoryAllocation ? STNTT_ENOMEM : STNTT_ECUDA,
                    std::string("cudaMalloc(workspace): ") + cudaGetErrorString(e));
    e = cudaMemset(static_cast<char *>(nb.buf.ptr) + bytes, 0, kWorkspaceTail);
    if (e != cudaSuccess) {
        cudaFree(nb.buf.ptr);
        return cuda_fail(ctx, e, "workspace tail");
    }
    nb.buf.bytes = bytes;
    std::lock_guard<std::mutex> g(ctx->mu);
    nb.last_use = ++ctx->ws_clock;
    auto ins = ctx->workspaces.emplace(s, nb);
    if (!ins.second) {  // another thread on the same stream stored one meanwhile
        if (ins.first->second.buf.bytes >= bytes) {
            cudaFree(nb.buf.ptr);
            *ptr = ins.first->second.buf.ptr;
            if (tail)
                *tail = static_cast<char *>(ins.first->second.buf.ptr) + ins.first->second.buf.bytes;
            return STNTT_OK;
        }
        // both were ordered on this stream: the smaller one is idle once the stream is
        cudaStreamSynchronize(s);
        cudaFree(ins.first->second.buf.ptr);
        ctx->mem -= ins.first->second.buf.bytes + kWorkspaceTail;
        ins.first->second = nb;
    }
    ctx->mem += bytes + kWorkspaceTail;
    *ptr = nb.buf.ptr;
    if (tail)
        *tail = static_cast<char *>(nb.buf.ptr) + bytes;
    return STNTT_OK;
}

int check_u32_args(stntt_ctx *ctx, uint32_t log_n, uint32_t p, uint32_t root) {
    if (log_n > 27)
        return fail(ctx, STNTT_EUNSUPPORTED, "log_n must be <= 27 for the 32-bit field");
    if (p < 2 || p >= (1u << 31))
        return fail(ctx, STNTT_EINVAL, "p must be a prime in [2, 2^31)");
    if (log_n > 0 && ((p - 1) % (1u << log_n)) != 0)
        return fail(ctx, STNTT_EINVAL, "p - 1 must be divisible by n");
    if (root == 0 || root >= p)
        return fail(ctx, STNTT_EINVAL, "root must lie in [1, p)");
    if (host_pow_mod(root, 1ull << log_n, p) != 1 || (log_n > 0 && host_pow_mod(root, 1ull << (log_n - 1), p) == 1))
        return fail(ctx, STNTT_EINVAL, "root is not a primitive n-th root of unity mod p");
    return STNTT_OK;
}

// A two-pass plan's passes as one launch of K-CTA clusters: CTA r takes n2/K
// columns in the first pass and n1/K rows in the second, exchanging through
// distributed shared memory. STNTT_EUNSUPPORTED when the shape does not fit
// (tile lengths 2^7..2^9 with 16 elements per thread, at most 32 KiB of the
// transform per CTA, the shared memory of a CTA, a prime without the lazy
// kernels).
struct ClusterShape {
    PassDesc d1, d2;
    uint32_t xoff = 0, xs = 0, log_k = 3;
    size_t smem = 0;
};

bool cluster_shape(const Plan &pl, uint32_t log_k, ClusterShape &cs) {
    if (pl.passes.size() != 2 || (pl.field != kFieldGL && pl.p >= (1u << 30)))
        return false;
    const PassDesc &p1 = pl.passes[0], &p2 = pl.passes[1];
    if ((p1.E != 16 && p1.E != 8) || p2.E != p1.E || p1.mode != kModeCol || p2.mode != kModeRow ||
        p1.full_off == ~0ull)
        return false;
    if (p1.E == 8 && (p1.logL + p2.logL < 16 || p1.logL < 7 || p2.logL < 7))
        return false;  // the 8-element cluster builds: 2^16- and 2^17-point splits
    // Up to 32 KiB per CTA of the cluster (256 KiB for 8 CTAs, 512 KiB for 16):
    // beyond that the cluster's SMs are compute-bound and the two-pass launches
    // were as fast or faster (measured: 8 CTAs at 2^16 Goldilocks, 2^17 32-bit).
    if ((pl.field == kFieldGL ? 8ull : 4ull) << pl.log_n > (32ull << (10 + log_k)))
        return false;
    const uint32_t L1 = p1.logL, L2 = p2.logL;
    if (L1 < 7 || L1 > 9 || L2 < 7 || L2 > 9 || L1 + L2 < 14 || L1 + L2 > 17)
        return false;
    cs.d1 = p1;
    cs.d2 = p2;
    cs.log_k = log_k;
    shape_pass(cs.d1, pl.field, 1ull << p1.logS, p1.E, 1u << (L2 - log_k));  // column limit: the sub-problem's columns
    shape_pass(cs.d2, pl.field, 1ull << 20, p1.E, 1u << (L1 - log_k));
    if (cs.d1.logC != L2 - log_k || cs.d2.logC != L1 - log_k || cs.d1.threads != cs.d2.threads)
        return false;
    const size_t esz = pl.field == kFieldGL ? 8 : 4;
    cs.xs = (1u << L1) + 1;  // odd: conflict-free column writes and row gathers
    const uint64_t work = std::max<uint64_t>((uint64_t)cs.d1.cs << cs.d1.logC, (uint64_t)cs.d2.cs << cs.d2.logC);
    cs.xoff = (uint32_t)((work + 3) & ~3ull);
    cs.smem = (cs.xoff + ((uint64_t)cs.xs << cs.d1.logC)) * esz;
    return cs.smem <= 200 * 1024;
}

// The cluster shape for this context: 16 CTAs where the device schedules them,
// else (or when 16 does not fit the plan) 8.
bool cluster_shape(const stntt_ctx *ctx, const Plan &pl, ClusterShape &cs) {
    return (ctx->cluster_log > kClusterLogSmall && cluster_shape(pl, ctx->cluster_log, cs)) ||
           cluster_shape(pl, kClusterLogSmall, cs);
}

// A two-pass plan's passes as one cooperative launch (coop.cuh): both passes
// reshaped to 8 points per thread and one block size (the larger pass's
// threads per line, at least 256). false when the shape does not fit (tiles
// of 2^8..2^11 points, 2^18..2^21-point transforms, no full four-step table,
// a prime with the lazy kernels).
struct CoopShape {
    PassDesc d1, d2;
    size_t smem = 0;
};

bool coop_shape(const Plan &pl, CoopShape &cs) {
    if (pl.passes.size() != 2 || (pl.field != kFieldGL && pl.p >= (1u << 30)))
        return false;
    const PassDesc &p1 = pl.passes[0], &p2 = pl.passes[1];
    if (p1.mode != kModeCol || p2.mode != kModeRow || p1.full_off != ~0ull || p1.logL < 8 || p1.logL > 11 ||
        p2.logL < 8 || p2.logL > 11 || pl.log_n < 18 || pl.log_n > 21)
        return false;
    const uint32_t u1 = (1u << p1.logL) / 8, u2 = (1u << p2.logL) / 8;
    const uint32_t T = std::max<uint32_t>(256, std::max(u1, u2));
    if (T > 512 || T / u1 > (1u << p1.logS) || T / u2 > (1u << (pl.log_n - p2.logL)))
        return false;
    cs.d1 = p1;
    cs.d2 = p2;
    cs.d1.vec = cs.d2.vec = 0;
    shape_pass(cs.d1, pl.field, 1ull << p1.logS, 8, T / u1);
    shape_pass(cs.d2, pl.field, 1ull << (pl.log_n - p2.logL), 8, T / u2);
    if (cs.d1.E != 8 || cs.d2.E != 8 || cs.d1.threads != T || cs.d2.threads != T)
        return false;
    cs.smem = std::max(cs.d1.smem_bytes, cs.d2.smem_bytes);
    return cs.smem <= 200 * 1024;
}

int run_coop(stntt_ctx *ctx, const Plan &pl, const void *in, void *out, uint64_t batch, cudaStream_t s) {
    CoopShape cs;
    if (ctx->coop_mode == 0 || !coop_shape(pl, cs))
        return STNTT_EUNSUPPORTED;
    const size_t bytes = (batch << pl.log_n) * (pl.field == kFieldGL ? 8 : 4);
    void *ws = nullptr, *tail = nullptr;
    const int rc = get_workspace(ctx, s, bytes, &ws, &tail);
    if (rc)
        return rc;
    const cudaError_t e = launch_coop(pl.field, cs.d1, cs.d2, pl.p, pl.d_tables, in, ws, out, batch, cs.smem, tail,
                                      ctx->d_err, s);
    if (e == cudaErrorNotSupported)
        return STNTT_EUNSUPPORTED;
    return e == cudaSuccess ? STNTT_OK : cuda_fail(ctx, e, "cooperative launch");
}

int run_cluster(stntt_ctx *ctx, const Plan &pl, const void *in, void *out, uint64_t batch, cudaStream_t s) {
    ClusterShape cs;
    if (!cluster_shape(ctx, pl, cs))
        return STNTT_EUNSUPPORTED;
    const cudaError_t e = launch_cluster(pl.field, cs.d1, cs.d2, pl.p, pl.d_tables, in, out, batch, cs.xoff, cs.xs,
                                         cs.smem, cs.log_k, s);
    if (e == cudaErrorNotSupported)
        return STNTT_EUNSUPPORTED;
    return e == cudaSuccess ? STNTT_OK : cuda_fail(ctx, e, "cluster launch");
}

// Run a plan: first pass reads `in`, last pass writes `out`.
int run_plan(stntt_ctx *ctx, const Plan &pl, const void *in, void *out, uint64_t batch, cudaStream_t s,
             const void *in2) {
    const size_t esz = pl.field == kFieldGL ? 8 : 4;
    const size_t bytes = (batch << pl.log_n) * esz;
    if (pl.passes.empty()) {  // n == 1: the identity
        if (in2) {
            cudaError_t e = launch_pointwise(pl.field, in, in2, out, (size_t)batch << pl.log_n, pl.p, s);
            return e == cudaSuccess ? STNTT_OK : cuda_fail(ctx, e, "pointwise launch");
        }
        if (in != out) {
            cudaError_t e = cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess)
                return cuda_fail(ctx, e, "cudaMemcpyAsync");
        }
        return STNTT_OK;
    }
    if (!in2 && pl.passes.size() == 2 && ((uint64_t)batch << pl.log_n) < kSmallCallElems) {
        // Small two-pass calls: both passes in one cluster launch (cluster.cuh)
        // up to 2^17 points, else in one cooperative launch (coop.cuh).
        int rc = run_cluster(ctx, pl, in, out, batch, s);
        if (rc == STNTT_EUNSUPPORTED)
            rc = run_coop(ctx, pl, in, out, batch, s);
        if (rc != STNTT_EUNSUPPORTED)
            return rc;
    }
    void *ws = nullptr;
    if (pl.passes.size() > 1) {
        int rc = get_workspace(ctx, s, bytes, &ws);
        if (rc)
            return rc;
    }
    const size_t K = pl.passes.size();
    const void *src = in;
    const PassDesc &p0 = pl.passes[0];
    if (in2 && p0.E != 16 && (1u << p0.logL) > p0.E) {  // no fused kernel for this shape: separate pointwise product
        cudaError_t e = launch_pointwise(pl.field, in, in2, out, (size_t)batch << pl.log_n, pl.p, s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "pointwise launch");
        src = out;
        in2 = nullptr;
    }
    for (size_t i = 0; i < K; ++i) {
        void *dst = (i + 1 == K) ? out : ws;
        cudaError_t e = launch_tile(pl.field, pl.passes[i], pl.p, pl.d_tables, src, dst, batch, s, i == 0 ? in2 : nullptr,
                                    ctx->d_err);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "tile kernel launch");
        src = dst;
    }
    return STNTT_OK;
}

// int32 wrap-around twiddle table of the reference: t_0 = 1,
// t_(i+1) = (t_i * root) % mod in 32-bit signed arithmetic (ntt_cpu.cpp:57-62).
int get_stage_table(stntt_ctx *ctx, uint32_t log_n, uint32_t p, uint32_t root, int wrap, const void **out) {
    std::lock_guard<std::mutex> g(ctx->mu);
    auto key = std::make_tuple(log_n, p, root, wrap);
    auto it = ctx->stage_tables.find(key);
    if (it != ctx->stage_tables.end()) {
        *out = it->second.ptr;
        return STNTT_OK;
    }
    const uint64_t half = log_n ? (1ull << (log_n - 1)) : 0;
    const size_t esz = wrap ? 4 : 8;
    DevBuf b;
    b.bytes = std::max<uint64_t>(half, 1) * esz;
    cudaError_t e = cudaMalloc(&b.ptr, b.bytes);
    if (e != cudaSuccess) {
        ctx->err = std::string("cudaMalloc(stage table): ") + cudaGetErrorString(e);
        return STNTT_ENOMEM;
    }
    if (wrap) {
        std::vector<int32_t> t(std::max<uint64_t>(half, 1));
        int32_t temp = 1;
        for (uint64_t i = 0; i < half; ++i) {
            t[i] = temp;
            temp = (int32_t)((uint32_t)temp * (uint32_t)root) % (int32_t)p;
        }
        e = cudaMemcpy(b.ptr, t.data(), b.bytes, cudaMemcpyHostToDevice);
    } else {
        e = launch_gen_powers(kFieldU32, b.ptr, half, root, 1, p, ctx->setup);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->setup);
    }
    if (e != cudaSuccess) {
        cudaFree(b.ptr);
        ctx->err = std::string("stage table: ") + cudaGetErrorString(e);
        return STNTT_ECUDA;
    }
    ctx->mem += b.bytes;
    ctx->stage_tables[key] = b;
    *out = b.ptr;
    return STNTT_OK;
}

// Radix-2 Stockham stages one launch each (debug / reference-compatible path).
int run_stages(stntt_ctx *ctx, uint32_t *d, uint32_t log_n, uint64_t batch, uint32_t p, uint32_t root,
               uint32_t nsteps, int wrap, cudaStream_t s) {
    if (nsteps == 0 || log_n == 0)
        return STNTT_OK;
    const void *tw = nullptr;
    int rc = get_stage_table(ctx, log_n, p, root, wrap, &tw);
    if (rc)
        return rc;
    const size_t bytes = (batch << log_n) * 4;
    void *ws = nullptr;
    rc = get_workspace(ctx, s, bytes, &ws);
    if (rc)
        return rc;
    void *a = d, *b = ws;
    for (uint32_t st = 0; st < nsteps; ++st) {
        cudaError_t e = launch_stage_u32(a, b, tw, log_n, st, p, wrap, batch, s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "stage kernel launch");
        std::swap(a, b);
    }
    if (a != d) {
        cudaError_t e = cudaMemcpyAsync(d, a, bytes, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "cudaMemcpyAsync");
    }
    return STNTT_OK;
}

// Device staging buffer for the host-buffer entry points (caller holds host_mu).
int host_stage(stntt_ctx *ctx, size_t bytes, void **ptr) {
    DevBuf &b = ctx->host_stage;
    if (b.bytes < bytes) {
        if (b.ptr) {
            cudaStreamSynchronize(ctx->host_stream);
            cudaFree(b.ptr);
            std::lock_guard<std::mutex> g(ctx->mu);
            ctx->mem -= b.bytes;
        }
        b.ptr = nullptr;
        b.bytes = 0;
        cudaError_t e = cudaMalloc(&b.ptr, bytes);
        if (e != cudaSuccess) {
            b.ptr = nullptr;
            return fail(ctx, STNTT_ENOMEM, std::string("cudaMalloc(host staging): ") + cudaGetErrorString(e));
        }
        b.bytes = bytes;
        std::lock_guard<std::mutex> g(ctx->mu);
        ctx->mem += bytes;
    }
    *ptr = b.ptr;
    return STNTT_OK;
}

// The end of a host-buffer call (caller holds host_mu): stop the device-work
// event, copy the result back, wait, and keep the device time between the two
// events for stntt_last_kernel_ms.
int host_finish(stntt_ctx *ctx, void *host, const void *dev, size_t bytes, cudaStream_t s) {
    cudaError_t e = cudaEventRecord(ctx->host_ev1, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "host copy out");
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, ctx->host_ev0, ctx->host_ev1);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaEventElapsedTime");
    ctx->host_kernel_ms = ms;
    return STNTT_OK;
}

int ctx_device(const stntt_ctx *ctx) { return ctx->device; }

// Drop every cached plan (caller holds ctx->mu; the device is idle).
void drop_plans(stntt_ctx *ctx) {
    for (auto &kv : ctx->plans) {
        if (kv.second->d_tables)
            cudaFree(kv.second->d_tables);
        ctx->mem -= kv.second->table_bytes;
    }
    ctx->plans.clear();
}

int release_workspace(stntt_ctx *ctx, cudaStream_t s) {
    StreamBuf b;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        auto it = ctx->workspaces.find(s);
        if (it == ctx->workspaces.end())
            return STNTT_OK;
        b = it->second;
        ctx->mem -= b.buf.bytes + kWorkspaceTail;
        ctx->workspaces.erase(it);
    }
    const cudaError_t e = cudaStreamSynchronize(s);
    if (b.buf.ptr)
        cudaFree(b.buf.ptr);
    return e == cudaSuccess ? STNTT_OK : cuda_fail(ctx, e, "release_stream: waiting for the stream");
}

}  // namespace sd

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int stntt_version(void) { return STNTT_VERSION; }

const char *stntt_status_string(int status) {
    switch (status) {
    case STNTT_OK: return "ok";
    case STNTT_EINVAL: return "invalid argument";
    case STNTT_ENOMEM: return "out of memory";
    case STNTT_ECUDA: return "CUDA error";
    case STNTT_ETIMEOUT: return "device wait timed out";
    case STNTT_EUNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

int stntt_init(stntt_ctx **out, int device) {
    if (!out)
        return STNTT_EINVAL;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return STNTT_EINVAL;
    auto ctx = new (std::nothrow) stntt_ctx();
    if (!ctx)
        return STNTT_ENOMEM;
    ctx->device = device;
    DeviceGuard g(device);
    // release whatever was created before a failing step
    auto undo = [ctx](int status) {
        if (ctx->d_err)
            cudaFree(ctx->d_err);
        if (ctx->host_ev0)
            cudaEventDestroy(ctx->host_ev0);
        if (ctx->host_ev1)
            cudaEventDestroy(ctx->host_ev1);
        if (ctx->setup)
            cudaStreamDestroy(ctx->setup);
        if (ctx->host_stream)
            cudaStreamDestroy(ctx->host_stream);
        delete ctx;
        return status;
    };
    if (g.err != cudaSuccess || cudaStreamCreateWithFlags(&ctx->setup, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->host_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->host_ev0) != cudaSuccess || cudaEventCreate(&ctx->host_ev1) != cudaSuccess)
        return undo(STNTT_ECUDA);
    if (cluster_max_size() >= 16)
        ctx->cluster_log = kClusterLogLarge;
    if (cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess || cudaMemset(ctx->d_err, 0, sizeof(int)) != cudaSuccess)
        return undo(STNTT_ENOMEM);
    // Load every kernel now: a lazy load at first use would stall the device
    // in the middle of a caller's stream of work. This also fails early when
    // the library holds no code for this GPU.
    if (preload_kernels() != cudaSuccess)
        return undo(STNTT_ECUDA);
    *out = ctx;
    return STNTT_OK;
}

int stntt_destroy(stntt_ctx *ctx) {
    if (!ctx)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    cudaDeviceSynchronize();
    for (auto &kv : ctx->plans)
        if (kv.second->d_tables)
            cudaFree(kv.second->d_tables);
    for (auto &kv : ctx->workspaces)
        if (kv.second.buf.ptr)
            cudaFree(kv.second.buf.ptr);
    for (auto &kv : ctx->stage_tables)
        if (kv.second.ptr)
            cudaFree(kv.second.ptr);
    if (ctx->host_stage.ptr)
        cudaFree(ctx->host_stage.ptr);
    if (ctx->d_err)
        cudaFree(ctx->d_err);
    if (ctx->setup)
        cudaStreamDestroy(ctx->setup);
    if (ctx->host_stream)
        cudaStreamDestroy(ctx->host_stream);
    if (ctx->host_ev0)
        cudaEventDestroy(ctx->host_ev0);
    if (ctx->host_ev1)
        cudaEventDestroy(ctx->host_ev1);
    delete ctx;
    return STNTT_OK;
}

const char *stntt_last_error(const stntt_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int stntt_mem_usage(const stntt_ctx *ctx, size_t *bytes) {
    if (!ctx || !bytes)
        return STNTT_EINVAL;
    *bytes = ctx->mem;
    return STNTT_OK;
}

int stntt_release_stream(stntt_ctx *ctx, stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    return release_workspace(ctx, (cudaStream_t)stream);
}

int stntt_last_kernel_ms(stntt_ctx *ctx, float *ms) {
    if (!ctx || !ms)
        return STNTT_EINVAL;
    std::lock_guard<std::mutex> hl(ctx->host_mu);
    *ms = ctx->host_kernel_ms;
    return STNTT_OK;
}

int stntt_find_params(uint64_t size, uint64_t min_mod, uint64_t *root, uint64_t *mod) {
    if (!root || !mod || size == 0 || min_mod == 0)
        return STNTT_EINVAL;
    uint64_t k = std::max<uint64_t>((min_mod - 1 + size - 1) / size, 1);
    uint64_t m = 0;
    for (;; ++k) {
        if (k > UINT64_MAX / size || k * size >= (1ull << 62))
            return STNTT_EUNSUPPORTED;
        if (is_prime_td(k * size + 1)) {
            m = k * size + 1;
            break;
        }
    }
    const uint64_t tot = m - 1;
    const std::vector<uint64_t> f = prime_factors(tot);
    uint64_t g = 0;
    for (uint64_t c = 1; c < m && !g; ++c) {
        if (host_pow_mod(c, tot, m) != 1 % m)
            continue;
        bool ok = true;
        for (uint64_t q : f)
            if (host_pow_mod(c, tot / q, m) == 1) {
                ok = false;
                break;
            }
        if (ok)
            g = c;
    }
    if (!g)
        return STNTT_EUNSUPPORTED;
    *mod = m;
    *root = host_pow_mod(g, tot / size, m);
    return STNTT_OK;
}

int stntt_find_params_device(uint64_t size, uint64_t min_mod, uint64_t *d_out, stntt_stream stream) {
    if (!d_out || size == 0 || min_mod == 0)
        return STNTT_EINVAL;
    if (size >= (1ull << 32) || min_mod >= (1ull << 32))
        return STNTT_EUNSUPPORTED;
    return launch_find_params(size, min_mod, d_out, (cudaStream_t)stream) == cudaSuccess ? STNTT_OK : STNTT_ECUDA;
}

int stntt_params_u32(uint32_t log_n, uint32_t *p, uint32_t *root) {
    if (!p || !root || log_n > 30)
        return STNTT_EINVAL;
    uint64_t r, m;
    int rc = stntt_find_params(1ull << log_n, 11, &r, &m);
    if (rc)
        return rc;
    if (m >= (1ull << 32))
        return STNTT_EUNSUPPORTED;
    *p = (uint32_t)m;
    *root = (uint32_t)r;
    return STNTT_OK;
}

int stntt_gl64_root(uint32_t log_n, uint64_t *root) {
    if (!root || log_n > 32)
        return STNTT_EINVAL;
    *root = host_gl_pow(7, (GL_P - 1) >> log_n);
    return STNTT_OK;
}

int stntt_prepare(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t p, uint32_t root, int dir) {
    if (!ctx || (dir != STNTT_FORWARD && dir != STNTT_INVERSE))
        return fail(ctx, STNTT_EINVAL, "bad context or direction");
    DeviceGuard g(ctx->device);
    const Plan *pl;
    if (field == STNTT_FIELD_GL64) {
        if (log_n > 32)
            return fail(ctx, STNTT_EUNSUPPORTED, "log_n must be <= 32 for Goldilocks");
        uint64_t r;
        stntt_gl64_root(log_n, &r);
        return get_plan(ctx, kFieldGL, log_n, 0, r, dir, &pl);
    }
    if (field != STNTT_FIELD_U32)
        return fail(ctx, STNTT_EINVAL, "unknown field");
    int rc = check_u32_args(ctx, log_n, p, root);
    if (rc)
        return rc;
    return get_plan(ctx, kFieldU32, log_n, p, root, dir, &pl);
}

int stntt_plan_info(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t p, uint32_t root, int dir,
                    uint32_t *passes, uint32_t *pass_logs) {
    if (!ctx || !passes)
        return STNTT_EINVAL;
    int rc = stntt_prepare(ctx, field, log_n, p, root, dir);
    if (rc)
        return rc;
    const Plan *pl;
    uint64_t r = root;
    if (field == STNTT_FIELD_GL64)
        stntt_gl64_root(log_n, &r);
    rc = get_plan(ctx, field == STNTT_FIELD_GL64 ? kFieldGL : kFieldU32, log_n, field == STNTT_FIELD_GL64 ? 0 : p,
                  r, dir, &pl);
    if (rc)
        return rc;
    *passes = (uint32_t)pl->passes.size();
    if (pass_logs)
        for (size_t i = 0; i < pl->passes.size() && i < 4; ++i)
            pass_logs[i] = pl->passes[i].logL;
    return STNTT_OK;
}

namespace {

int set_plan_for(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs,
                 const uint32_t *elems, const uint32_t *cols, int kind) {
    if (!ctx || !pass_logs || npasses == 0 || npasses > (kind == kPlanBatched ? 2u : 3u))
        return fail(ctx, STNTT_EINVAL, "set_plan: bad arguments");
    if (field != STNTT_FIELD_U32 && field != STNTT_FIELD_GL64)
        return fail(ctx, STNTT_EINVAL, "set_plan: unknown field");
    PlanSpec s;
    uint32_t sum = 0;
    for (uint32_t i = 0; i < npasses; ++i) {
        const uint32_t lg = pass_logs[i], e = elems ? elems[i] : 0, c = cols ? cols[i] : 0;
        if (lg == 0 || lg > 13)
            return fail(ctx, STNTT_EINVAL, "set_plan: each pass length must be 2^1..2^13");
        const uint32_t eb = e & ~(STNTT_PASS_VEC | STNTT_PASS_CLUSTER);
        const bool vec_e = (e & STNTT_PASS_VEC) != 0;
        if (vec_e ? (eb != 0 && eb != 4 && eb != 8 && eb != 16) : (eb != 0 && eb != 8 && eb != 16 && eb != 32))
            return fail(ctx, STNTT_EINVAL,
                        "set_plan: elems must be 0, 8, 16 or 32 (STNTT_PASS_VEC with 0, 4, 8 or 16)");
        if ((e & STNTT_PASS_CLUSTER) && (!(e & STNTT_PASS_VEC) || (eb != 0 && eb != 8)))
            return fail(ctx, STNTT_EINVAL, "set_plan: STNTT_PASS_CLUSTER goes with STNTT_PASS_VEC and 8 points per line");
        if (c & (c - 1))
            return fail(ctx, STNTT_EINVAL, "set_plan: cols must be 0 or a power of two");
        s.logs.push_back(lg);
        s.elems.push_back(e);
        s.cols.push_back(c);
        sum += lg;
    }
    if (sum != log_n)
        return fail(ctx, STNTT_EINVAL, "set_plan: pass lengths must multiply to 2^log_n");
    const int f = field == STNTT_FIELD_GL64 ? kFieldGL : kFieldU32;
    DeviceGuard g(ctx->device);
    cudaDeviceSynchronize();  // plans about to be freed may be in use
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->specs[{f, log_n, kind}] = s;
    for (auto it = ctx->plans.begin(); it != ctx->plans.end();) {
        if (it->first.field == f && it->first.log_n == log_n) {
            if (it->second->d_tables)
                cudaFree(it->second->d_tables);
            ctx->mem -= it->second->table_bytes;
            it = ctx->plans.erase(it);
        } else {
            ++it;
        }
    }
    return STNTT_OK;
}

}  // namespace

int stntt_call_info(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t batch, uint32_t p, uint32_t root, int dir,
                    uint32_t *launches, uint32_t *pass_logs) {
    if (!ctx || !launches || batch == 0)
        return STNTT_EINVAL;
    if (dir != STNTT_FORWARD && dir != STNTT_INVERSE)
        return fail(ctx, STNTT_EINVAL, "call_info: bad direction");
    int f;
    uint64_t r = root;
    if (field == STNTT_FIELD_GL64) {
        if (log_n > 32)
            return fail(ctx, STNTT_EUNSUPPORTED, "log_n must be <= 32 for Goldilocks");
        f = kFieldGL;
        p = 0;
        stntt_gl64_root(log_n, &r);
    } else if (field == STNTT_FIELD_U32) {
        const int rc = check_u32_args(ctx, log_n, p, root);
        if (rc)
            return rc;
        f = kFieldU32;
    } else {
        return fail(ctx, STNTT_EINVAL, "call_info: unknown field");
    }
    DeviceGuard g(ctx->device);
    const Plan *pl;
    const int rc = get_plan(ctx, f, log_n, p, r, dir, &pl, ((uint64_t)batch << log_n) < kSmallCallElems);
    if (rc)
        return rc;
    ClusterShape cs;
    CoopShape co;
    const bool small = ((uint64_t)batch << log_n) < kSmallCallElems;
    const bool one = small && (cluster_shape(ctx, *pl, cs) || (ctx->coop_mode != 0 && coop_shape(*pl, co)));
    *launches = one ? 1u : (uint32_t)pl->passes.size();
    if (pass_logs)
        for (size_t i = 0; i < pl->passes.size() && i < 4; ++i)
            pass_logs[i] = pl->passes[i].logL;
    return STNTT_OK;
}

int stntt_set_plan(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs,
                   const uint32_t *elems, const uint32_t *cols) {
    return set_plan_for(ctx, field, log_n, npasses, pass_logs, elems, cols, kPlanAll);
}

int stntt_set_plan_small(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs,
                         const uint32_t *elems, const uint32_t *cols) {
    return set_plan_for(ctx, field, log_n, npasses, pass_logs, elems, cols, kPlanSmall);
}

int stntt_set_plan_batched(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs) {
    if (npasses == 1 && pass_logs && pass_logs[0] < 4)
        return fail(ctx, STNTT_EINVAL, "set_plan_batched: passes must be at least 2^4 points");
    if (npasses == 2 && pass_logs && (pass_logs[0] < 4 || pass_logs[1] < 4))
        return fail(ctx, STNTT_EINVAL, "set_plan_batched: passes must be at least 2^4 points");
    // a work item of a two-pass job holds 8192 elements of that one job
    if (npasses == 2 && log_n < kBatchTileLog)
        return fail(ctx, STNTT_EINVAL, "set_plan_batched: two passes need at least 2^13 points");
    return set_plan_for(ctx, field, log_n, npasses, pass_logs, nullptr, nullptr, kPlanBatched);
}

int stntt_device_key(int device, char *buf, size_t len) {
    if (!buf || len == 0)
        return STNTT_EINVAL;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return STNTT_EINVAL;
    int drv = 0;
    cudaDriverGetVersion(&drv);
    snprintf(buf, len, "%s|%d|%d|%d.%d", prop.name, prop.multiProcessorCount, drv, prop.major, prop.minor);
    return STNTT_OK;
}

int stntt_clear_plans(stntt_ctx *ctx) {
    if (!ctx)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->specs.clear();
    drop_plans(ctx);
    return STNTT_OK;
}

int stntt_set_tma(stntt_ctx *ctx, int mode) {
    if (!ctx || mode < -1 || mode > 1)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->tma_mode != mode) {
        ctx->tma_mode = mode;
        drop_plans(ctx);
    }
    return STNTT_OK;
}

int stntt_set_coop(stntt_ctx *ctx, int mode) {
    if (!ctx || mode < 0 || mode > 1)
        return STNTT_EINVAL;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->coop_mode = mode;
    return STNTT_OK;
}

int stntt_device_status(stntt_ctx *ctx) {
    if (!ctx)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    int flag = 0;
    cudaError_t e = cudaMemcpy(&flag, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && flag)
        e = cudaMemset(ctx->d_err, 0, sizeof(int));
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "reading the device error word");
    if (flag) {
        // a bounded wait ran out: clear every stream's barrier words, which a
        // cooperative launch that gave up may have left mid-count
        cudaDeviceSynchronize();
        std::lock_guard<std::mutex> lk(ctx->mu);
        for (auto &kv : ctx->workspaces)
            cudaMemset(static_cast<char *>(kv.second.buf.ptr) + kv.second.buf.bytes, 0, kWorkspaceTail);
        ctx->err = "a device-side wait gave up (a TMA-staged copy or the grid barrier of a cooperative launch); "
                   "that call's output is incomplete";
        return STNTT_ETIMEOUT;
    }
    return STNTT_OK;
}

int stntt_selftest_tma_timeout(stntt_ctx *ctx, uint32_t spin_limit) {
    if (!ctx || spin_limit == 0)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    cudaError_t e = launch_tma_selftest(ctx->d_err, spin_limit, ctx->setup);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->setup);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "TMA wait self-test");
    return stntt_device_status(ctx);
}

int stntt_ntt_u32_oop(stntt_ctx *ctx, const uint32_t *d_in, uint32_t *d_out, uint32_t log_n, uint32_t batch,
                      uint32_t p, uint32_t root, int dir, stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    if ((!d_in || !d_out) && batch)
        return fail(ctx, STNTT_EINVAL, "null data pointer");
    if (dir != STNTT_FORWARD && dir != STNTT_INVERSE)
        return fail(ctx, STNTT_EINVAL, "dir must be STNTT_FORWARD or STNTT_INVERSE");
    int rc = check_u32_args(ctx, log_n, p, root);
    if (rc)
        return rc;
    if (batch == 0)
        return STNTT_OK;
    DeviceGuard g(ctx->device);
    const Plan *pl;
    rc = get_plan(ctx, kFieldU32, log_n, p, root, dir, &pl, ((uint64_t)batch << log_n) < kSmallCallElems);
    if (rc)
        return rc;
    return run_plan(ctx, *pl, d_in, d_out, batch, (cudaStream_t)stream);
}

int stntt_ntt_u32(stntt_ctx *ctx, uint32_t *d_data, uint32_t log_n, uint32_t batch, uint32_t p, uint32_t root,
                  int dir, uint32_t flags, stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    if (flags & ~STNTT_FLAG_REF_WRAP)
        return fail(ctx, STNTT_EINVAL, "unknown flags");
    if (flags & STNTT_FLAG_REF_WRAP) {
        if (dir != STNTT_FORWARD)
            return fail(ctx, STNTT_EINVAL, "STNTT_FLAG_REF_WRAP supports the forward transform only");
        return stntt_ntt_u32_steps(ctx, d_data, log_n, batch, p, root, log_n, flags, stream);
    }
    return stntt_ntt_u32_oop(ctx, d_data, d_data, log_n, batch, p, root, dir, stream);
}

int stntt_ntt_u32_steps(stntt_ctx *ctx, uint32_t *d_data, uint32_t log_n, uint32_t batch, uint32_t p,
                        uint32_t root, uint32_t nsteps, uint32_t flags, stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    if (!d_data && batch)
        return fail(ctx, STNTT_EINVAL, "null data pointer");
    if (flags & ~STNTT_FLAG_REF_WRAP)
        return fail(ctx, STNTT_EINVAL, "unknown flags");
    if (nsteps > log_n)
        return fail(ctx, STNTT_EINVAL, "nsteps must be <= log_n");
    const int wrap = (flags & STNTT_FLAG_REF_WRAP) ? 1 : 0;
    if (wrap) {  // the reference accepts any int modulus / root; only the size limits apply
        if (log_n > 30 || p < 2 || p >= (1u << 31))
            return fail(ctx, STNTT_EINVAL, "REF_WRAP needs log_n <= 30 and 2 <= p < 2^31");
    } else {
        int rc = check_u32_args(ctx, log_n, p, root);
        if (rc)
            return rc;
    }
    if (batch == 0)
        return STNTT_OK;
    DeviceGuard g(ctx->device);
    return run_stages(ctx, d_data, log_n, batch, p, root, nsteps, wrap, (cudaStream_t)stream);
}

int stntt_ntt_gl64_oop(stntt_ctx *ctx, const uint64_t *d_in, uint64_t *d_out, uint32_t log_n, uint32_t batch,
                       int dir, stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    if ((!d_in || !d_out) && batch)
        return fail(ctx, STNTT_EINVAL, "null data pointer");
    if (dir != STNTT_FORWARD && dir != STNTT_INVERSE)
        return fail(ctx, STNTT_EINVAL, "dir must be STNTT_FORWARD or STNTT_INVERSE");
    if (log_n > 32)
        return fail(ctx, STNTT_EUNSUPPORTED, "log_n must be <= 32 for Goldilocks");
    if (batch == 0)
        return STNTT_OK;
    DeviceGuard g(ctx->device);
    uint64_t r;
    stntt_gl64_root(log_n, &r);
    const Plan *pl;
    int rc = get_plan(ctx, kFieldGL, log_n, 0, r, dir, &pl, ((uint64_t)batch << log_n) < kSmallCallElems);
    if (rc)
        return rc;
    return run_plan(ctx, *pl, d_in, d_out, batch, (cudaStream_t)stream);
}

int stntt_ntt_gl64(stntt_ctx *ctx, uint64_t *d_data, uint32_t log_n, uint32_t batch, int dir, stntt_stream stream) {
    return stntt_ntt_gl64_oop(ctx, d_data, d_data, log_n, batch, dir, stream);
}

int stntt_ntt_stockham_host(stntt_ctx *ctx, int32_t *vec, int32_t size, int32_t root, int32_t mod, int32_t batches,
                            int32_t nsteps, uint32_t flags) {
    if (!ctx)
        return STNTT_EINVAL;
    if (size <= 0 || (size & (size - 1)))
        return fail(ctx, STNTT_EINVAL, "size (" + std::to_string(size) + ") must be a power of 2");
    if (!vec || batches < 0)
        return fail(ctx, STNTT_EINVAL, "null vector or negative batch count");
    if (mod < 2)
        return fail(ctx, STNTT_EINVAL, "mod must be >= 2");
    if (batches == 0)
        return STNTT_OK;
    const uint32_t log_n = ilog2((uint64_t)size);
    if (nsteps > (int32_t)log_n)
        return fail(ctx, STNTT_EINVAL, "nsteps must be <= log2(size)");
    const bool wrap = (flags & STNTT_FLAG_REF_WRAP) != 0;
    const size_t count = (size_t)size * (size_t)batches;
    std::vector<int32_t> staged;
    const int32_t *src = vec;
    if (!wrap) {  // the exact field transform takes canonical residues
        staged.assign(vec, vec + count);
        for (auto &v : staged) {
            int32_t r = v % mod;
            v = r >= 0 ? r : r + mod;
        }
        src = staged.data();
    }
    DeviceGuard g(ctx->device);
    std::lock_guard<std::mutex> hl(ctx->host_mu);
    void *dv = nullptr;
    int rc = host_stage(ctx, count * 4, &dv);
    if (rc)
        return rc;
    uint32_t *d = static_cast<uint32_t *>(dv);
    cudaStream_t s = ctx->host_stream;
    cudaError_t e = cudaMemcpyAsync(d, src, count * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "host copy in");
    e = cudaEventRecord(ctx->host_ev0, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaEventRecord");
    if (nsteps >= 0 && (uint32_t)nsteps < log_n)
        rc = stntt_ntt_u32_steps(ctx, d, log_n, (uint32_t)batches, (uint32_t)mod, (uint32_t)root, (uint32_t)nsteps,
                                 flags, s);
    else
        rc = stntt_ntt_u32(ctx, d, log_n, (uint32_t)batches, (uint32_t)mod, (uint32_t)root, STNTT_FORWARD, flags, s);
    if (rc) {
        cudaStreamSynchronize(s);
        return rc;
    }
    return host_finish(ctx, vec, d, count * 4, s);
}

int stntt_ntt_gl64_host(stntt_ctx *ctx, uint64_t *vec, uint32_t log_n, uint32_t batch, int dir) {
    if (!ctx)
        return STNTT_EINVAL;
    if (!vec && batch)
        return fail(ctx, STNTT_EINVAL, "null vector");
    if (log_n > 32)
        return fail(ctx, STNTT_EUNSUPPORTED, "log_n must be <= 32 for Goldilocks");
    if (batch == 0)
        return STNTT_OK;
    const size_t count = (size_t)batch << log_n;
    DeviceGuard g(ctx->device);
    std::lock_guard<std::mutex> hl(ctx->host_mu);
    void *dv = nullptr;
    int rc = host_stage(ctx, count * 8, &dv);
    if (rc)
        return rc;
    cudaStream_t s = ctx->host_stream;
    cudaError_t e = cudaMemcpyAsync(dv, vec, count * 8, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "host copy in");
    e = cudaEventRecord(ctx->host_ev0, s);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaEventRecord");
    rc = stntt_ntt_gl64(ctx, static_cast<uint64_t *>(dv), log_n, batch, dir, s);
    if (rc) {
        cudaStreamSynchronize(s);
        return rc;
    }
    return host_finish(ctx, vec, dv, count * 8, s);
}

int stntt_ntt_batch_per_call(stntt_ctx *ctx, const stntt_job *jobs, size_t njobs, stntt_stream stream) {
    if (!ctx || (!jobs && njobs))
        return STNTT_EINVAL;
    for (size_t i = 0; i < njobs; ++i) {
        const stntt_job &j = jobs[i];
        int rc;
        if (j.field == STNTT_FIELD_GL64)
            rc = stntt_ntt_gl64(ctx, static_cast<uint64_t *>(j.data), j.log_n, 1, (int)j.dir, stream);
        else if (j.field == STNTT_FIELD_U32)
            rc = stntt_ntt_u32(ctx, static_cast<uint32_t *>(j.data), j.log_n, 1, j.p, j.root, (int)j.dir, 0, stream);
        else
            rc = fail(ctx, STNTT_EINVAL, "unknown field in job");
        if (rc)
            return rc;
    }
    return STNTT_OK;
}


int stntt_pointwise_mul_u32(const uint32_t *d_a, const uint32_t *d_b, uint32_t *d_out, size_t count, uint32_t p,
                            stntt_stream stream) {
    if ((!d_a || !d_b || !d_out) && count)
        return STNTT_EINVAL;
    if (p < 2 || p >= (1u << 31))
        return STNTT_EINVAL;
    if (!count)
        return STNTT_OK;
    return launch_pointwise(kFieldU32, d_a, d_b, d_out, count, p, (cudaStream_t)stream) == cudaSuccess ? STNTT_OK
                                                                                                      : STNTT_ECUDA;
}

int stntt_pointwise_mul_gl64(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_out, size_t count,
                             stntt_stream stream) {
    if ((!d_a || !d_b || !d_out) && count)
        return STNTT_EINVAL;
    if (!count)
        return STNTT_OK;
    return launch_pointwise(kFieldGL, d_a, d_b, d_out, count, 0, (cudaStream_t)stream) == cudaSuccess ? STNTT_OK
                                                                                                     : STNTT_ECUDA;
}

}  // extern "C"
namespace sd {
int polymul_impl(stntt_ctx *ctx, int field, const void *a, const void *b, void *out, uint32_t log_n,
                        uint32_t p, uint64_t root, cudaStream_t s) {
    const size_t esz = field == kFieldGL ? 8 : 4;
    const size_t bytes = ((size_t)1 << log_n) * esz;
    const Plan *fwd, *inv;
    const bool small = (1ull << log_n) < kSmallCallElems;
    int rc = get_plan(ctx, field, log_n, p, root, STNTT_FORWARD, &fwd, small);
    if (!rc)
        rc = get_plan(ctx, field, log_n, p, root, STNTT_INVERSE, &inv, small);
    if (rc)
        return rc;
    // workspace: [pass scratch n][second operand n]
    void *ws = nullptr;
    rc = get_workspace(ctx, s, 2 * bytes, &ws);
    if (rc)
        return rc;
    void *tb = static_cast<char *>(ws) + bytes;
    // b first: `out` may alias `b`
    if ((rc = run_plan(ctx, *fwd, b, tb, 1, s)))
        return rc;
    if ((rc = run_plan(ctx, *fwd, a, out, 1, s)))
        return rc;
    // the pointwise product happens inside the inverse's first pass (it
    // multiplies the two forward outputs as it loads them)
    return run_plan(ctx, *inv, out, out, 1, s, tb);
}
}  // namespace sd
extern "C" {

int stntt_polymul_u32(stntt_ctx *ctx, const uint32_t *d_a, const uint32_t *d_b, uint32_t *d_out, uint32_t log_n,
                      uint32_t p, uint32_t root, stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    if (!d_a || !d_b || !d_out)
        return fail(ctx, STNTT_EINVAL, "null pointer");
    int rc = check_u32_args(ctx, log_n, p, root);
    if (rc)
        return rc;
    DeviceGuard g(ctx->device);
    return polymul_impl(ctx, kFieldU32, d_a, d_b, d_out, log_n, p, root, (cudaStream_t)stream);
}

int stntt_polymul_gl64(stntt_ctx *ctx, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_out, uint32_t log_n,
                       stntt_stream stream) {
    if (!ctx)
        return STNTT_EINVAL;
    if (!d_a || !d_b || !d_out)
        return fail(ctx, STNTT_EINVAL, "null pointer");
    if (log_n > 32)
        return fail(ctx, STNTT_EUNSUPPORTED, "log_n must be <= 32 for Goldilocks");
    DeviceGuard g(ctx->device);
    uint64_t r;
    stntt_gl64_root(log_n, &r);
    return polymul_impl(ctx, kFieldGL, d_a, d_b, d_out, log_n, 0, r, (cudaStream_t)stream);
}

int stntt_fill_uniform_u32(uint32_t *d_out, size_t count, uint64_t seed, uint32_t p, stntt_stream stream) {
    if ((!d_out && count) || p < 2)
        return STNTT_EINVAL;
    if (!count)
        return STNTT_OK;
    return launch_fill_uniform(kFieldU32, d_out, count, seed, p, (cudaStream_t)stream) == cudaSuccess ? STNTT_OK
                                                                                                      : STNTT_ECUDA;
}

int stntt_measure_gl64_butterfly_rate(int device, double *rate) {
    if (!rate)
        return STNTT_EINVAL;
    DeviceGuard g(device);
    if (g.err != cudaSuccess)
        return STNTT_EINVAL;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const unsigned blocks = (unsigned)sms * 8, threads = 256;
    const int reps = 100;
    uint64_t *d = nullptr;
    if (cudaMalloc(&d, (size_t)blocks * threads * 8) != cudaSuccess)
        return STNTT_ENOMEM;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    float ms = 0;
    if (e == cudaSuccess)
        e = launch_gl_probe(d, blocks, 4, s);  // warm-up
    if (e == cudaSuccess)
        e = cudaEventRecord(e0, s);
    if (e == cudaSuccess)
        e = launch_gl_probe(d, blocks, reps, s);
    if (e == cudaSuccess)
        e = cudaEventRecord(e1, s);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(e1);
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (s)
        cudaStreamDestroy(s);
    cudaFree(d);
    if (e != cudaSuccess || ms <= 0)
        return STNTT_ECUDA;
    *rate = (double)blocks * threads * reps * 32.0 / (ms * 1e-3);  // 32 butterflies per repetition
    return STNTT_OK;
}

int stntt_fill_uniform_gl64(uint64_t *d_out, size_t count, uint64_t seed, stntt_stream stream) {
    if (!d_out && count)
        return STNTT_EINVAL;
    if (!count)
        return STNTT_OK;
    return launch_fill_uniform(kFieldGL, d_out, count, seed, 0, (cudaStream_t)stream) == cudaSuccess ? STNTT_OK
                                                                                                     : STNTT_ECUDA;
}

}  // extern "C"

// ===========================================================================
// Persistent batched launch (batch.cuh): host-side work list
// ===========================================================================
namespace {

struct BatchItemH {  // layout of stntt::BatchItem
    uint32_t args, wait_job, wait_count, signal_job;
    uint64_t blk;
};
static_assert(sizeof(BatchItemH) == 24, "BatchItem layout");
struct BatchCtlH {
    unsigned long long next;
    unsigned int error, timeouts;
};

constexpr unsigned kDefaultSpinLimit = 5000000;  // polls of ~200 ns: about one second

struct BatchPart {
    int field = 0;
    bool lazy = false;  // 32-bit field: every job's p < 2^30
    void *d_buf = nullptr;
    size_t args_off = 0, items_off = 0, counters_off = 0, ctl_off = 0, ptr_off = 0, bytes = 0;
    unsigned long long nitems = 0;
    uint32_t ncounters = 0;
    size_t smem = 0;
    unsigned grid = 0;
};

size_t args_size(int field) { return field == kFieldGL ? batch_args_size_gl64() : batch_args_size_u32(); }
void args_fill(int field, const PassDesc &d, uint32_t p, const void *t, const unsigned long long *ip,
               const unsigned long long *op, uint64_t total, void *dst) {
    if (field == kFieldGL)
        batch_args_fill_gl64(d, p, t, ip, op, total, dst);
    else
        batch_args_fill_u32(d, p, t, ip, op, total, dst);
}

// 512-thread tile shape for the persistent kernel: 16 elements per thread,
// C = 8192 / L columns or rows.
// Goldilocks items of two-pass jobs in the vector-lines layout: on unless
// STNTT_BATCH_VEC=0 (read once).
bool batch_vec_items() {
    static const bool v = [] {
        const char *e = getenv("STNTT_BATCH_VEC");
        return !(e && e[0] == '0');
    }();
    return v;
}

void batch_shape(PassDesc &d, int field) {
    const uint32_t L = 1u << d.logL;
    d.E = 16;
    const uint32_t U = L / 16, C = (1u << kBatchTileLog) / L;
    d.logC = ilog2(C);
    d.threads = C * U;
    d.cs = column_stride(field, L, C, U, d.tfast);
    d.smem_bytes = (size_t)C * d.cs * (field == kFieldGL ? 8 : 4);
}

}  // namespace

struct stntt_batch {
    stntt_ctx *ctx = nullptr;
    std::vector<BatchPart> parts;
    std::vector<stntt_job> fallback;
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    unsigned spin_limit = kDefaultSpinLimit;
};

namespace {

struct ClassKey {
    uint32_t log_n, dir, p, root;
    bool operator<(const ClassKey &o) const {
        return std::tie(log_n, dir, p, root) < std::tie(o.log_n, o.dir, o.p, o.root);
    }
};

int build_part(stntt_ctx *ctx, stntt_batch *bt, int field, const std::vector<const stntt_job *> &jobs,
               size_t &scratch_cursor) {
    std::map<ClassKey, std::vector<const stntt_job *>> classes;
    bool lazy = field == kFieldU32;  // the part's kernel: the lazy 32-bit field when every p < 2^30
    bool lazy8 = lazy;               // and its vector-lines items when every p < 2^29 (8p < 2^32)
    for (const stntt_job *j : jobs) {
        classes[{j->log_n, j->dir, field == kFieldGL ? 0u : j->p, field == kFieldGL ? 0u : j->root}].push_back(j);
        if (field == kFieldU32 && j->p >= (1u << 30))
            lazy = false;
        if (field == kFieldU32 && j->p >= (1u << 29))
            lazy8 = false;
    }
    const size_t asz = args_size(field);
    std::vector<unsigned char> args;                   // TileArgs, by value
    std::vector<unsigned long long> ptrs;              // per-class data / scratch pointer arrays
    std::vector<size_t> ptr_fix;                       // args records whose pointer fields are ptr offsets
    std::vector<BatchItemH> phaseA, phaseB;
    uint32_t njob2 = 0;
    size_t smem = 0;
    struct PendingArgs {
        PassDesc d;
        uint32_t p;
        const void *tables;
        size_t in_off, out_off;
        uint64_t total;
    };
    std::vector<PendingArgs> pend;
    for (auto &kv : classes) {
        const ClassKey &ck = kv.first;
        const auto &cj = kv.second;
        const Plan *pl = nullptr;
        uint64_t root = ck.root;
        if (field == kFieldGL)
            stntt_gl64_root(ck.log_n, &root);
        int rc = get_plan(ctx, field, ck.log_n, ck.p, root, (int)ck.dir, &pl, kPlanBatched);
        if (rc)
            return rc;
        if (field == kFieldGL)  // the batched kernel serves the two standard roots (TileArgs::pow2)
            for (const PassDesc &d : pl->passes)
                if (d.pow2 == 0)
                    return fail(ctx, STNTT_EUNSUPPORTED, "batch: Goldilocks root without a kernel build");
        const size_t J = cj.size();
        const size_t data_off = ptrs.size();
        for (const stntt_job *j : cj)
            ptrs.push_back((unsigned long long)(uintptr_t)j->data);
        if (pl->passes.size() == 1) {
            PassDesc d = pl->passes[0];
            d.tfast = 1;
            d.vec = 0;  // packed single-pass items keep the 16-points-per-thread layout (TileArgs::vecl = 0)
            batch_shape(d, field);
            smem = std::max(smem, d.smem_bytes);
            const uint32_t a_idx = (uint32_t)pend.size();
            pend.push_back({d, ck.p, pl->d_tables, data_off, data_off, (uint64_t)J});
            const uint64_t C = 1ull << d.logC;
            for (uint64_t blk = 0; blk * C < J; ++blk)
                phaseA.push_back({a_idx, ~0u, 0u, ~0u, blk});
        } else {
            // two passes: data -> scratch -> data
            const size_t scr_off = ptrs.size();
            const uint64_t n = 1ull << ck.log_n;
            for (size_t i = 0; i < J; ++i) {
                ptrs.push_back((unsigned long long)(uintptr_t)(static_cast<char *>(bt->d_scratch) + scratch_cursor));
                scratch_cursor += n * (field == kFieldGL ? 8 : 4);
            }
            PassDesc d0 = pl->passes[0], d1 = pl->passes[1];
            d0.tfast = 0;
            d1.tfast = 0;
            batch_shape(d0, field);
            batch_shape(d1, field);
            smem = std::max({smem, d0.smem_bytes, d1.smem_bytes});
            // The items run the vector-lines steps (batch_item_vec) when every
            // job's data is 16-byte aligned, both passes are 2^4..2^11 points
            // and the column pass has a full four-step table (16-byte aligned:
            // an even entry offset from the 256-byte aligned table
            // allocation); for the 32-bit field only in a part of the lazy
            // field whose primes leave the steps' headroom (every p < 2^29).
            const uint32_t V = field == kFieldGL ? 2 : 4, w = field == kFieldGL ? 8 : 4;
            bool vec = (field == kFieldGL || lazy8) && batch_vec_items() && d0.full_off != ~0ull &&
                       (d0.full_off & 1u) == 0 && !d0.full_mont && d0.logL >= 4 && d0.logL <= 11 && d1.logL >= 4 &&
                       d1.logL <= 11;
            for (const stntt_job *j : cj)
                vec = vec && ((uintptr_t)j->data & 15u) == 0;
            d0.vec = d1.vec = 0;  // TileArgs::vecl: set below only where the checks above hold
            if (vec) {
                d0.vec = d1.vec = V;
                const uint32_t lv = V == 2 ? 1 : 2;
                smem = std::max({smem, vec_smem(V, 13 - d0.logL - lv, d0.logL, w),
                                 vec_smem(V, 13 - d1.logL - lv, d1.logL, w)});
            }
            const uint32_t a0 = (uint32_t)pend.size();
            pend.push_back({d0, ck.p, pl->d_tables, data_off, scr_off, (uint64_t)J << (ck.log_n - d0.logL)});
            const uint32_t a1 = (uint32_t)pend.size();
            pend.push_back({d1, ck.p, pl->d_tables, scr_off, data_off, (uint64_t)J << (ck.log_n - d1.logL)});
            const uint64_t per0 = 1ull << (ck.log_n - d0.logL - d0.logC);  // items per job, pass 0
            const uint64_t per1 = 1ull << (ck.log_n - d1.logL - d1.logC);
            for (size_t i = 0; i < J; ++i) {
                const uint32_t job = njob2++;
                for (uint64_t k = 0; k < per0; ++k)
                    phaseA.push_back({a0, ~0u, 0u, job, i * per0 + k});
                for (uint64_t k = 0; k < per1; ++k)
                    phaseB.push_back({a1, job, (uint32_t)per0, ~0u, i * per1 + k});
            }
        }
    }
    BatchPart part;
    part.field = field;
    part.lazy = lazy;
    part.nitems = phaseA.size() + phaseB.size();
    part.ncounters = std::max<uint32_t>(njob2, 1);
    part.smem = smem;
    // device layout: args | items | ptrs | counters | ctl
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    part.args_off = 0;
    part.items_off = al(pend.size() * asz);
    part.ptr_off = al(part.items_off + part.nitems * sizeof(BatchItemH));
    part.counters_off = al(part.ptr_off + ptrs.size() * sizeof(unsigned long long));
    part.ctl_off = al(part.counters_off + part.ncounters * sizeof(unsigned int));
    part.bytes = al(part.ctl_off + sizeof(BatchCtlH));
    cudaError_t e = cudaMalloc(&part.d_buf, part.bytes);
    if (e != cudaSuccess)
        return fail(ctx, STNTT_ENOMEM, std::string("cudaMalloc(batch work list): ") + cudaGetErrorString(e));
    bt->parts.push_back(part);
    BatchPart &P = bt->parts.back();
    std::vector<unsigned char> host(P.bytes, 0);
    char *dbase = static_cast<char *>(P.d_buf);
    const unsigned long long *dptrs = reinterpret_cast<const unsigned long long *>(dbase + P.ptr_off);
    for (size_t i = 0; i < pend.size(); ++i)
        args_fill(field, pend[i].d, pend[i].p, pend[i].tables, dptrs + pend[i].in_off, dptrs + pend[i].out_off,
                  pend[i].total, host.data() + i * asz);
    std::memcpy(host.data() + P.items_off, phaseA.data(), phaseA.size() * sizeof(BatchItemH));
    std::memcpy(host.data() + P.items_off + phaseA.size() * sizeof(BatchItemH), phaseB.data(),
                phaseB.size() * sizeof(BatchItemH));
    std::memcpy(host.data() + P.ptr_off, ptrs.data(), ptrs.size() * sizeof(unsigned long long));
    e = cudaMemcpy(P.d_buf, host.data(), P.bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "batch work list upload");
    int bps = 0;
    e = field == kFieldGL ? batch_prepare_gl64(P.smem, &bps)
                          : (P.lazy ? batch_prepare_u32l(P.smem, &bps) : batch_prepare_u32(P.smem, &bps));
    if (e != cudaSuccess || bps < 1)
        return fail(ctx, STNTT_ECUDA, "batch kernel does not fit on an SM");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    P.grid = (unsigned)std::min<unsigned long long>(P.nitems ? P.nitems : 1, (unsigned long long)sms * bps);
    return STNTT_OK;
}

}  // namespace

extern "C" {

int stntt_batch_create(stntt_ctx *ctx, const stntt_job *jobs, size_t njobs, stntt_batch **out) {
    if (!ctx || !out || (!jobs && njobs))
        return STNTT_EINVAL;
    *out = nullptr;
    DeviceGuard g(ctx->device);
    std::vector<const stntt_job *> by_field[2];
    auto bt = std::make_unique<stntt_batch>();
    bt->ctx = ctx;
    size_t scratch_total = 0;
    for (size_t i = 0; i < njobs; ++i) {
        const stntt_job &j = jobs[i];
        if (j.dir != STNTT_FORWARD && j.dir != STNTT_INVERSE)
            return fail(ctx, STNTT_EINVAL, "job " + std::to_string(i) + ": bad direction");
        if (!j.data)
            return fail(ctx, STNTT_EINVAL, "job " + std::to_string(i) + ": null data");
        int f;
        uint32_t passes = 0;
        if (j.field == STNTT_FIELD_GL64) {
            if (j.log_n > 32)
                return fail(ctx, STNTT_EUNSUPPORTED, "job " + std::to_string(i) + ": log_n > 32");
            f = kFieldGL;
        } else if (j.field == STNTT_FIELD_U32) {
            int rc = check_u32_args(ctx, j.log_n, j.p, j.root);
            if (rc)
                return rc;
            f = kFieldU32;
        } else {
            return fail(ctx, STNTT_EINVAL, "job " + std::to_string(i) + ": unknown field");
        }
        size_t scratch_need = 0;
        if (j.log_n >= 4) {
            const Plan *pl;
            uint64_t root = j.root;
            if (f == kFieldGL)
                stntt_gl64_root(j.log_n, &root);
            int rc = get_plan(ctx, f, j.log_n, f == kFieldGL ? 0 : j.p, root, (int)j.dir, &pl, kPlanBatched);
            if (rc)
                return rc;
            passes = (uint32_t)pl->passes.size();
            for (const PassDesc &d : pl->passes)
                if (d.logL < 4)
                    passes = 99;  // the persistent kernel's tiles are at least 16 long
            if (passes == 2 && j.log_n < kBatchTileLog)
                passes = 99;  // a two-pass work item holds 8192 elements of one job
            if (passes == 2)
                scratch_need = ((size_t)1 << j.log_n) * (f == kFieldGL ? 8 : 4);
        }
        if (j.log_n >= 4 && passes <= 2) {
            by_field[f].push_back(&j);
            scratch_total += scratch_need;
        } else {
            bt->fallback.push_back(j);
        }
    }
    if (scratch_total) {
        cudaError_t e = cudaMalloc(&bt->d_scratch, scratch_total);
        if (e != cudaSuccess)
            return fail(ctx, STNTT_ENOMEM, std::string("cudaMalloc(batch scratch): ") + cudaGetErrorString(e));
        bt->scratch_bytes = scratch_total;
    }
    size_t cursor = 0;
    for (int f = 0; f < 2; ++f) {
        if (by_field[f].empty())
            continue;
        int rc = build_part(ctx, bt.get(), f, by_field[f], cursor);
        if (rc) {
            stntt_batch_destroy(bt.release());
            return rc;
        }
    }
    *out = bt.release();
    return STNTT_OK;
}

int stntt_batch_launch(stntt_batch *b, stntt_stream stream) {
    if (!b)
        return STNTT_EINVAL;
    stntt_ctx *ctx = b->ctx;
    DeviceGuard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    for (BatchPart &P : b->parts) {
        char *base = static_cast<char *>(P.d_buf);
        cudaError_t e = cudaMemsetAsync(base + P.counters_off, 0, P.bytes - P.counters_off, s);
        if (e == cudaSuccess)
            e = P.field == kFieldGL
                    ? batch_launch_gl64(base + P.args_off, base + P.items_off, P.nitems,
                                        reinterpret_cast<unsigned int *>(base + P.counters_off), base + P.ctl_off,
                                        P.smem, P.grid, b->spin_limit, s)
                    : (P.lazy ? batch_launch_u32l : batch_launch_u32)(
                          base + P.args_off, base + P.items_off, P.nitems,
                          reinterpret_cast<unsigned int *>(base + P.counters_off), base + P.ctl_off, P.smem, P.grid,
                          b->spin_limit, s);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "batch launch");
    }
    if (!b->fallback.empty())
        return stntt_ntt_batch_per_call(ctx, b->fallback.data(), b->fallback.size(), stream);
    return STNTT_OK;
}

int stntt_batch_status(stntt_batch *b) {
    if (!b)
        return STNTT_EINVAL;
    DeviceGuard g(b->ctx->device);
    for (BatchPart &P : b->parts) {
        BatchCtlH c;
        cudaError_t e = cudaMemcpy(&c, static_cast<char *>(P.d_buf) + P.ctl_off, sizeof(c), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            return cuda_fail(b->ctx, e, "batch status");
        if (c.error)
            return fail(b->ctx, STNTT_ETIMEOUT,
                        std::to_string(c.timeouts) + " batch work item(s) gave up waiting for their first pass");
    }
    return STNTT_OK;
}

int stntt_batch_info(const stntt_batch *b, size_t *items, uint32_t *grid, size_t *fallback) {
    if (!b)
        return STNTT_EINVAL;
    size_t it = 0;
    uint32_t gr = 0;
    for (const BatchPart &P : b->parts) {
        it += P.nitems;
        gr += P.grid;
    }
    if (items)
        *items = it;
    if (grid)
        *grid = gr;
    if (fallback)
        *fallback = b->fallback.size();
    return STNTT_OK;
}

int stntt_batch_destroy(stntt_batch *b) {
    if (!b)
        return STNTT_EINVAL;
    DeviceGuard g(b->ctx->device);
    cudaDeviceSynchronize();
    for (BatchPart &P : b->parts)
        if (P.d_buf)
            cudaFree(P.d_buf);
    if (b->d_scratch)
        cudaFree(b->d_scratch);
    delete b;
    return STNTT_OK;
}

int stntt_ntt_batch(stntt_ctx *ctx, const stntt_job *jobs, size_t njobs, stntt_stream stream) {
    stntt_batch *b = nullptr;
    int rc = stntt_batch_create(ctx, jobs, njobs, &b);
    if (rc)
        return rc;
    rc = stntt_batch_launch(b, stream);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        rc = e == cudaSuccess ? stntt_batch_status(b) : cuda_fail(ctx, e, "batch execution");
    }
    stntt_batch_destroy(b);
    return rc;
}

int stntt_selftest_wait_timeout(stntt_ctx *ctx, uint32_t spin_limit) {
    if (!ctx || spin_limit == 0)
        return STNTT_EINVAL;
    DeviceGuard g(ctx->device);
    stntt_batch b;
    b.ctx = ctx;
    b.spin_limit = spin_limit;
    BatchPart P;
    P.field = kFieldGL;
    P.nitems = 1;
    P.ncounters = 1;
    P.smem = 0;
    P.grid = 1;
    const size_t asz = args_size(kFieldGL);
    P.args_off = 0;
    P.items_off = 256 * ((asz + 255) / 256);
    P.ptr_off = P.items_off + 256;
    P.counters_off = P.ptr_off + 256;
    P.ctl_off = P.counters_off + 256;
    P.bytes = P.ctl_off + 256;
    cudaError_t e = cudaMalloc(&P.d_buf, P.bytes);
    if (e != cudaSuccess)
        return fail(ctx, STNTT_ENOMEM, "selftest allocation");
    std::vector<unsigned char> host(P.bytes, 0);
    // one item that waits for a job counter nothing increments
    BatchItemH it{0u, 0u, 1u, ~0u, 0ull};
    std::memcpy(host.data() + P.items_off, &it, sizeof(it));
    int bps = 0;
    e = cudaMemcpy(P.d_buf, host.data(), P.bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = batch_prepare_gl64(0, &bps);
    if (e != cudaSuccess) {
        cudaFree(P.d_buf);
        return cuda_fail(ctx, e, "selftest setup");
    }
    b.parts.push_back(P);
    int rc = stntt_batch_launch(&b, nullptr);
    if (!rc) {
        e = cudaStreamSynchronize(nullptr);
        rc = e == cudaSuccess ? stntt_batch_status(&b) : cuda_fail(ctx, e, "selftest run");
    }
    cudaFree(P.d_buf);
    b.parts.clear();
    return rc;
}

}  // extern "C"
