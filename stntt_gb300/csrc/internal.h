// internal.h -- interface between the host planner (api.cu) and the per-field
// kernel translation units (kernels_u32.cu, kernels_gl64.cu). Not installed.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace stntt {

enum : int { kFieldU32 = 0, kFieldGL = 1 };
enum : uint32_t { kModeCol = 0, kModeRow = 1 };  // tile pass kinds (tile.cuh)
// Column passes over sub-problems of 2^14..2^20 points read their four-step
// twiddle from a full table (at most 8 MB, so it stays in L2 across the
// batch and the sub-problems); larger ones, whose table would stream from
// HBM on the store path, keep the two-level lookup. Calls of fewer than 2^22
// elements use full tables only up to 2^17 points: a lone 2^20-point call
// would read its 8 MB table from HBM once per call, as many bytes as its data
// (measured on GB300, Goldilocks 2^20 forward + inverse with L2 flushed
// between steps: 84.5 us with the full table, 77.8 us without). Passes of
// small calls in the vector-lines build, whose table loads are 16 bytes wide,
// take full tables up to 2^21 points (Goldilocks 2^20 forward, best plan:
// 31.8 us against 32.9; 2^21: 51.4 against 55.4).
constexpr uint32_t kFullTwiddleMinLog = 14, kFullTwiddleMaxLog = 20, kFullTwiddleMaxLogSmall = 17;
constexpr uint32_t kFullTwiddleMaxLogSmallVec = 21;
// Passes in the vector-lines build (tile_v.cuh) of calls of 2^22+ elements
// use full tables up to 2^26-point sub-problems (see build_plan).
constexpr uint32_t kFullTwiddleMaxLogVec = 26;
// 32-bit vector-lines column passes of calls of 2^22+ elements: Montgomery
// table entries from 2^17-point sub-problems on (api.cu, full_mont_min_log)
constexpr uint32_t kFullMontMinLog = 17;
// One-launch transforms: 16-CTA clusters (non-portable size) where the device
// schedules them, else 8; up to 2^(15 + log2 K) bytes per transform.
constexpr uint32_t kClusterLogSmall = 3, kClusterLogLarge = 4;

// One HBM pass of a transform plan (see tile.cuh for the meaning of the fields).
struct PassDesc {
    uint32_t logL = 0, logC = 0, E = 16, mode = 1, do_scale = 0, tfast = 1, h = 0;
    uint32_t logN = 0, logM = 0, logS = 0, logN1 = 0, logN2 = 0;
    uint32_t cs = 0;          // shared-memory column stride, elements
    uint32_t threads = 0;     // threads per CTA
    size_t smem_bytes = 0;
    uint64_t tw_off = 0, lo_off = 0, hi_off = 0;  // table offsets, in table entries
    uint64_t full_off = ~0ull;  // COL: w_M^(col*pos) for every (pos, col), laid out like the data; ~0 = none
    uint64_t wR[8] = {};      // raw twiddle entries (u32: {w, w'} packed little-endian)
    uint64_t scale = 0;       // raw twiddle entry
    uint32_t tma = 0;         // 1: run as the TMA-staged persistent kernel where the pass allows it (tma.cuh)
    // The vector-lines build (tile_v.cuh) of this pass, when vec != 0: vec
    // lines per thread (4 four-byte or 2 eight-byte), vE points per line per
    // thread, 2^vlogG line groups per CTA, vthreads threads and vsmem bytes of
    // shared memory. The fields above
    // keep the plain build's shape, which runs where the vector build cannot
    // (unaligned pointers, a prime of 2^30 or more).
    uint32_t vec = 0, vE = 16, vlogG = 0, vthreads = 0;
    size_t vsmem = 0;
    // 32-bit vector-lines column pass: the table at full_off holds M 4-byte
    // Montgomery entries (w * 2^32 mod p) instead of Shoup pairs; the plain
    // build, which cannot read it, takes the two-level tables instead.
    uint32_t full_mont = 0, pinv = 0;
    // Goldilocks: 1 when the transform's root is the standard forward root
    // 7^((p-1)/n) (then w_16 = 2^156), 2 when it is its inverse (w_16 =
    // 2^36), else 0; the kernels built on FieldGLPow2 (shift-only internal
    // twiddles) serve only passes with 1 or 2.
    uint32_t pow2 = 0;
    // Vector-lines cluster build (tile_vc.cuh), when vcl != 0: each line's
    // DFT over the 2^vcl CTAs of a thread-block cluster, first phase of
    // 2^vlog1 points; vlogG, vthreads and vsmem then describe one CTA.
    uint32_t vcl = 0, vlog1 = 0;
};

// ---- launchers (return the CUDA error of the launch) ----------------------
// err: the context's device error word; the TMA-staged kernel (tma.cuh) runs
// only when it is given (its bounded waits report there).
cudaError_t launch_tile(int field, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                        uint64_t batch, cudaStream_t s, const void *in2 = nullptr, int *err = nullptr);
// The TMA-staged kernel with no copy issued, so that its first wait runs out
// after spin_limit polls and sets *err (self-test of the bounded wait).
cudaError_t launch_tma_selftest(int *err, uint32_t spin_limit, cudaStream_t s);
// Polls of an mbarrier before the TMA-staged kernel gives up (about a second).
constexpr uint32_t kTmaSpinLimit = 1u << 22;
// out[i] = scale * base^i, i < count, as twiddle entries (u32: Shoup pairs).
cudaError_t launch_gen_powers(int field, void *out, uint64_t count, uint64_t base, uint64_t scale, uint32_t p,
                              cudaStream_t s);
// Both passes of a two-pass plan as one thread-block-cluster launch (cluster.cuh);
// cudaErrorNotSupported when this plan or prime cannot use it.
cudaError_t launch_cluster(int field, const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                           const void *in, void *out, uint64_t batch, uint32_t xoff, uint32_t xs, size_t smem,
                           uint32_t log_k, cudaStream_t s);
// Largest cluster the current device schedules for the cluster kernels (8 or 16).
int cluster_max_size();
// The vector-lines build of a pass (tile_v.cuh); cudaErrorNotSupported when
// the pass or its pointers do not allow it (the caller then runs the plain one).
cudaError_t launch_tile_vec(int field, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                            uint64_t batch, cudaStream_t s);
cudaError_t preload_vec();
// The vector-lines cluster build of a pass (tile_vc.cuh, d.vcl != 0).
cudaError_t launch_tile_vc(int field, const PassDesc &d, uint32_t p, const void *tables, const void *in, void *out,
                           uint64_t batch, cudaStream_t s);
cudaError_t preload_vc();
// Both passes of a two-pass plan in one cooperative launch (coop.cuh): d1 the
// column pass into ws, d2 the row pass into out, with equal block sizes; bar:
// the stream's zero-initialised barrier words; err: the device error word.
// cudaErrorNotSupported when the shape is not instantiated or not resident.
cudaError_t launch_coop(int field, const PassDesc &d1, const PassDesc &d2, uint32_t p, const void *tables,
                        const void *in, void *ws, void *out, uint64_t batch, size_t smem, void *bar, int *err,
                        cudaStream_t s);
// out[pos * 2^logS + col] = w_M^(col * pos) for count = M entries, from the
// two-level tables lo (w_M^e, e < 2^h) and hi (s * w_M^(e 2^h)).
cudaError_t launch_gen_four_step(int field, void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS,
                                 uint64_t count, uint32_t p, cudaStream_t s);
// The same table for the 32-bit field in Montgomery form: out (4-byte entries)
// = w_M^(col * pos) * 2^32 mod p, from the Shoup-pair tables lo / hi.
cudaError_t launch_gen_four_step_mont(void *out, const void *lo, const void *hi, uint32_t h, uint32_t logS,
                                      uint64_t count, uint32_t p, cudaStream_t s);
cudaError_t launch_pointwise(int field, const void *a, const void *b, void *out, size_t count, uint32_t p,
                             cudaStream_t s);
cudaError_t launch_fill_uniform(int field, void *out, size_t count, uint64_t seed, uint32_t p, cudaStream_t s);
// One radix-2 Stockham DIF stage (src/ntt/ntt_cpu.cpp:66-79) over `batch`
// transforms. wrap != 0: the reference's int32 arithmetic with its wrapped
// twiddle table (int32 entries); else exact with a Shoup-pair table.
cudaError_t launch_stage_u32(const void *in, void *out, const void *tw, uint32_t log_n, uint32_t stage, uint32_t p,
                             int wrap, uint64_t batch, cudaStream_t s);
cudaError_t launch_copy_scale(int field, const void *in, void *out, size_t count, uint64_t scale_tw, uint32_t p,
                              cudaStream_t s);

// Load every kernel of the library on the current device (see
// preload_tiles_t); run once per device when a context is created.
cudaError_t preload_kernels();

// Host modular helpers
uint64_t host_pow_mod(uint64_t b, uint64_t e, uint64_t m);
uint64_t host_gl_mul(uint64_t a, uint64_t b);
uint64_t host_gl_pow(uint64_t b, uint64_t e);
// Twiddle entry for a value (u32: {w, floor(w * 2^32 / p)} packed; gl: w)
uint64_t host_tw_entry(int field, uint64_t w, uint32_t p);

}  // namespace stntt
