/*
 * stntt.h -- C ABI of the GB300-native stNTT library (libstntt.so).
 *
 * Number-theoretic transforms on one NVIDIA GB300 (sm_103a), natural order in
 * and out, over two fields:
 *   - the reference's per-size 32-bit prime: p = k*n + 1 (the smallest such
 *     prime >= min_mod) with root g^((p-1)/n), g the smallest generator
 *     (findParams, src/ntt/ntt_util.cpp:10-49); any prime p < 2^31 with a
 *     primitive n-th root is accepted;
 *   - Goldilocks, p = 2^64 - 2^32 + 1, root 7^((p-1)/n).
 *
 * Conventions
 *   - Forward:  X[k] = sum_j x[j] * root^(j*k) mod p        (nttStockham)
 *   - Inverse:  x[j] = n^-1 * sum_k X[k] * root^(-j*k) mod p
 *   - Device-pointer calls are asynchronous on the caller's stream
 *     (a cudaStream_t passed as `stream`; NULL = legacy default stream).
 *   - The caller owns every data buffer. A context owns its twiddle tables,
 *     plans and per-stream workspaces. Every function returns a status and
 *     never exits the process; stntt_last_error() gives the message.
 *   - The first call for a given (field, size, root, direction) builds its
 *     twiddle tables and synchronises an internal stream: make that first
 *     call (or stntt_prepare) before capturing a stream into a CUDA graph.
 *   - Input residues must be canonical (< p) unless stated otherwise.
 *
 * Thread safety: one context may be shared by several host threads (its caches
 * are locked); calls on different streams use different workspaces.
 */
#ifndef STNTT_H
#define STNTT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STNTT_VERSION 1

typedef enum stntt_status {
    STNTT_OK = 0,
    STNTT_EINVAL = 1,       /* bad argument (reference: std::invalid_argument) */
    STNTT_ENOMEM = 2,       /* device or host allocation failed */
    STNTT_ECUDA = 3,        /* a CUDA runtime call failed (reference: CCErr -> exit) */
    STNTT_ETIMEOUT = 4,     /* a bounded device-side wait gave up */
    STNTT_EUNSUPPORTED = 5, /* size / field combination outside the supported range */
} stntt_status;

typedef enum stntt_dir { STNTT_FORWARD = 0, STNTT_INVERSE = 1 } stntt_dir;
typedef enum stntt_field { STNTT_FIELD_U32 = 0, STNTT_FIELD_GL64 = 1 } stntt_field;

/* flags for the 32-bit field */
#define STNTT_FLAG_REF_WRAP 0x1u /* reproduce the reference's int32 wrap-around arithmetic
                                    (forward only; equals the reference CPU bit for bit) */

typedef struct stntt_ctx stntt_ctx;
typedef void *stntt_stream; /* a cudaStream_t */

/* ---- context -------------------------------------------------------------- */
/* Replaces the reference's process-global device state (__constant__ twiddles
 * and global_twiddles, src/cuda/ntt/implementations/common.cuh:7-9). */
int stntt_init(stntt_ctx **ctx, int device);
int stntt_destroy(stntt_ctx *ctx);
const char *stntt_last_error(const stntt_ctx *ctx);
const char *stntt_status_string(int status);
int stntt_version(void);
/* Bytes of device memory the context currently holds (tables + workspaces). */
int stntt_mem_usage(const stntt_ctx *ctx, size_t *bytes);
/* Free the scratch the context keeps for `stream` (the buffer between HBM
 * passes, one per stream a multi-pass transform ran on), after waiting for the
 * stream's work. A caller that makes a stream per request releases it before
 * destroying the stream; the context also keeps at most 16 such buffers and
 * frees the least recently used one (after waiting for its stream) when a
 * 17th stream appears. No counterpart in the reference, which allocates and
 * frees a double buffer on every autoNtt call (src/cuda/ntt/ntt_kernel.cuh:157-160). */
int stntt_release_stream(stntt_ctx *ctx, stntt_stream stream);

/* ---- parameters ------------------------------------------------------------- */
/* findParams(size, min_mod) -> (root, mod): src/ntt/ntt_util.cpp:10-14
 * (findModulus :16-27, findPrimitiveRoot :29-34, findGenerator :36-42). */
int stntt_find_params(uint64_t size, uint64_t min_mod, uint64_t *root, uint64_t *mod);
/* The same search on the device, asynchronous on `stream`, for moduli below
 * 2^32: writes d_out[0] = root, d_out[1] = mod, d_out[2] = status (STNTT_OK,
 * or STNTT_EUNSUPPORTED when no prime k*size + 1 >= min_mod lies below 2^32).
 * No host round trip, so parameters can be produced inside a CUDA graph.
 * Returns STNTT_EUNSUPPORTED for size or min_mod >= 2^32. */
int stntt_find_params_device(uint64_t size, uint64_t min_mod, uint64_t *d_out, stntt_stream stream);
/* findParams(2^log_n, 11), the call every reference caller makes
 * (src/main.cu:37, src/bench.cu:35, src/tests/cuda/ntt/st_ntt_test.cu:20). */
int stntt_params_u32(uint32_t log_n, uint32_t *p, uint32_t *root);
/* Goldilocks root of unity of order 2^log_n (log_n <= 32): 7^((p-1)/2^log_n). */
int stntt_gl64_root(uint32_t log_n, uint64_t *root);

/* Build (or look up) the twiddle tables and plan for a transform, on an
 * internal stream, and wait for them. Optional: the transform calls do it on
 * first use. For STNTT_FIELD_GL64, p and root are ignored. */
int stntt_prepare(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t p, uint32_t root, int dir);

/* Shape of the plan stntt_prepare builds: the number of HBM passes (kernel
 * launches per transform) and log2 of each pass's tile length (up to 4). */
int stntt_plan_info(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t p, uint32_t root, int dir,
                    uint32_t *passes, uint32_t *pass_logs);

/* What one call of this shape does: the number of kernel launches per
 * transform call (1 when both passes of a small two-pass plan run as one
 * thread-block-cluster launch) and log2 of each pass's tile length (up to 4),
 * for the plan a call with this batch uses. */
int stntt_call_info(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t batch, uint32_t p, uint32_t root, int dir,
                    uint32_t *launches, uint32_t *pass_logs);

/* elems flag: run the pass with the vector-lines build (V adjacent lines per
 * thread, 16-byte loads and stores; passes of multi-pass plans with tiles of
 * 2^7..2^10 points, 16 points per line, or 8 with elems = 8 | STNTT_PASS_VEC);
 * cols then gives the lines per CTA (4 or 8 times V, V = 4 for the 32-bit
 * field and 2 for Goldilocks). */
#define STNTT_PASS_VEC 0x100u
/* elems flag, with STNTT_PASS_VEC and 8 points per line: the vector-lines
 * cluster build for passes of 2^11..2^13 points (each line's DFT spread over
 * the 8 CTAs of a thread-block cluster through distributed shared memory),
 * which makes two-pass plans of 2^22..2^26 points possible; cols gives the
 * lines per cluster (4 or 8 times V). */
#define STNTT_PASS_CLUSTER 0x200u

/* Override the plan for one (field, log_n): npasses HBM passes (1..4) with
 * tile lengths 2^pass_logs[i] (summing to log_n, each <= 13; npasses <= 3), elements per
 * thread elems[i] (16 or 32, or 8 for tiles of 2^7..2^11 points; 0 = default; may carry
 * STNTT_PASS_VEC) and columns per CTA cols[i] (a power
 * of two; 0 = default). Drops cached plans of that size. The autotuner
 * (stntt_gb300/tune.py) drives this and stores its choices on disk.
 * stntt_clear_plans() restores the built-in defaults for every size. */
int stntt_set_plan(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs,
                   const uint32_t *elems, const uint32_t *cols);
/* The same for small calls only: transforms of this size in calls of fewer
 * than 2^22 elements in all (batch * n), such as single requests, where the
 * best shape fills the GPU with more, narrower tiles. Without it small calls
 * use the plan above. No counterpart in the reference (it has one launch
 * shape per n, src/cuda/ntt/ntt_kernel.cuh:31-39). */
int stntt_set_plan_small(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs,
                         const uint32_t *elems, const uint32_t *cols);
/* The pass split (1 or 2 passes, each of 2^4..2^13 points) a job of this size
 * takes inside the persistent batched launch (stntt_batch_create,
 * stntt_ntt_batch), whose tiles are 8192 elements with 16 per thread; tuned
 * separately because that kernel's best split differs from a plain call's.
 * Extends the reference's manual block-size sweep (src/bench.cu:88-91). */
int stntt_set_plan_batched(stntt_ctx *ctx, int field, uint32_t log_n, uint32_t npasses, const uint32_t *pass_logs);
int stntt_clear_plans(stntt_ctx *ctx);
/* "name|SM count|driver version|compute capability" of a device: the key
 * under which tuned plans are cached. */
int stntt_device_key(int device, char *buf, size_t len);

/* ---- transforms on device buffers ------------------------------------------ */
/* In place, `batch` contiguous transforms of 2^log_n elements.
 * Replaces cuda::ntt::autoNtt<n>(NttArgs) (src/cuda/ntt/ntt_kernel.cuh:153-200)
 * and the kernels it launches (stNttRadix2, stNttRadix2Adaptive,
 * sttNttGlobalRadix2). Supported: log_n in [0, 27] with p < 2^31.
 * flags: STNTT_FLAG_REF_WRAP (dir must be STNTT_FORWARD). */
int stntt_ntt_u32(stntt_ctx *ctx, uint32_t *d_data, uint32_t log_n, uint32_t batch, uint32_t p, uint32_t root,
                  int dir, uint32_t flags, stntt_stream stream);
/* Goldilocks, in place. The Goldilocks driver sttNttGoldilocks
 * (src/cuda/ntt/implementations/st_ntt_goldilocks.cuh:198-225) is a
 * non-functional scaffold in the reference; this is its working counterpart.
 * Supported: log_n in [0, 32]. */
int stntt_ntt_gl64(stntt_ctx *ctx, uint64_t *d_data, uint32_t log_n, uint32_t batch, int dir, stntt_stream stream);
/* Out-of-place variants: d_in is not modified (may equal d_out). */
int stntt_ntt_u32_oop(stntt_ctx *ctx, const uint32_t *d_in, uint32_t *d_out, uint32_t log_n, uint32_t batch,
                      uint32_t p, uint32_t root, int dir, stntt_stream stream);
int stntt_ntt_gl64_oop(stntt_ctx *ctx, const uint64_t *d_in, uint64_t *d_out, uint32_t log_n, uint32_t batch,
                       int dir, stntt_stream stream);
/* The first `nsteps` radix-2 Stockham stages only (nsteps <= log_n), the
 * reference's std::optional<int> nsteps hook (src/ntt/ntt_cpu.h:8). A debug
 * path: one launch per stage. flags as for stntt_ntt_u32. */
int stntt_ntt_u32_steps(stntt_ctx *ctx, uint32_t *d_data, uint32_t log_n, uint32_t batch, uint32_t p,
                        uint32_t root, uint32_t nsteps, uint32_t flags, stntt_stream stream);

/* ---- host-buffer convenience (copies in, transforms, copies out; synchronous) */
/* Mirrors nttStockham(int *vec, int size, int root, int mod, nsteps) and its
 * batched overload (src/ntt/ntt_cpu.h:8-9, ntt_cpu.cpp:46-90): in place on a
 * host int array. nsteps < 0 means all stages. Without STNTT_FLAG_REF_WRAP the
 * result is the exact field NTT (equal to the reference for n <= 2^13); with
 * it, equal to the reference at every n. */
int stntt_ntt_stockham_host(stntt_ctx *ctx, int32_t *vec, int32_t size, int32_t root, int32_t mod,
                            int32_t batches, int32_t nsteps, uint32_t flags);
int stntt_ntt_gl64_host(stntt_ctx *ctx, uint64_t *vec, uint32_t log_n, uint32_t batch, int dir);
/* Device time, in milliseconds, of the last host-buffer call on this context
 * (stntt_ntt_stockham_host or stntt_ntt_gl64_host): CUDA events recorded
 * after the copy in and before the copy out, around the transform's kernels.
 * The value cuda::ntt::autoNtt<n> returns as its kernel time
 * (src/cuda/ntt/ntt_kernel.cuh:167,187-191; stored as gpuTime by
 * src/bench.cu:48-50). */
int stntt_last_kernel_ms(stntt_ctx *ctx, float *ms);

/* ---- uneven batches ----------------------------------------------------------- */
typedef struct stntt_job {
    uint32_t field; /* stntt_field */
    uint32_t log_n;
    uint32_t dir;   /* stntt_dir */
    uint32_t p;     /* STNTT_FIELD_U32 only */
    uint32_t root;  /* STNTT_FIELD_U32 only */
    uint32_t reserved;
    void *data;     /* device pointer, 2^log_n elements, transformed in place */
} stntt_job;

/* Many independent transforms of uneven sizes, fields and directions in one
 * persistent launch per field (jobs with log_n < 4 or needing three HBM
 * passes run as ordinary launches after it). Extends the reference's uniform
 * `batches` packing (src/cuda/ntt/ntt_kernel.cuh:31-39). Synchronous: builds
 * the work list, launches on `stream`, waits, and returns STNTT_ETIMEOUT if a
 * bounded device-side wait gave up. Job buffers must not overlap. */
int stntt_ntt_batch(stntt_ctx *ctx, const stntt_job *jobs, size_t njobs, stntt_stream stream);
/* Same jobs, one launch sequence per job (the comparison baseline). */
int stntt_ntt_batch_per_call(stntt_ctx *ctx, const stntt_job *jobs, size_t njobs, stntt_stream stream);

/* Reusable batch (for CUDA graphs): create builds twiddle tables, the work
 * list and a private scratch buffer (synchronous, not inside a capture);
 * launch only zeroes its counters and launches (capturable, repeatable);
 * status reads the device error flag once the stream has completed. */
typedef struct stntt_batch stntt_batch;
int stntt_batch_create(stntt_ctx *ctx, const stntt_job *jobs, size_t njobs, stntt_batch **out);
int stntt_batch_launch(stntt_batch *b, stntt_stream stream);
int stntt_batch_status(stntt_batch *b);
/* items: work items of the persistent launches; grid: their total blocks;
 * fallback: jobs run as ordinary launches. */
int stntt_batch_info(const stntt_batch *b, size_t *items, uint32_t *grid, size_t *fallback);
int stntt_batch_destroy(stntt_batch *b);
/* Launch the persistent kernel on one work item whose dependency nothing
 * satisfies, with the given poll limit; returns STNTT_ETIMEOUT when the
 * kernel's bounded wait gave up and reported it (the context stays usable). */
int stntt_selftest_wait_timeout(stntt_ctx *ctx, uint32_t spin_limit);

/* ---- TMA-staged passes ---------------------------------------------------------- */
/* Passes of 2^7..2^12-point tiles can run as a persistent kernel whose tiles
 * are copied into shared memory by the Tensor Memory Accelerator (a copy of
 * the next tile overlaps the current tile's work). No counterpart in the
 * reference, whose kernels load each element with its own instruction
 * (st_ntt_global_radix2.cuh:8-86). mode: -1 = built-in choice per pass
 * (the default), 0 = never, 1 = wherever the pass allows it. Drops cached plans. */
int stntt_set_tma(stntt_ctx *ctx, int mode);
/* STNTT_ETIMEOUT when a staged pass on this context gave up waiting for a copy
 * (after about a second) since the last call -- its output is then
 * incomplete -- else STNTT_OK. Reads a device word: synchronise the streams
 * that ran the transforms first. Clears the word. */
/* Small calls (fewer than 2^22 elements) of a two-pass plan of 2^18..2^21
 * points may run both passes in one cooperative launch (a grid-wide barrier
 * between the passes, bounded like every device-side wait): 1 where the shape
 * fits, 0 (default) never, i.e. two launches, which measured faster on GB300
 * at every such size. No counterpart in the reference, which launches every
 * stage separately and synchronises the host between them
 * (src/cuda/ntt/implementations/st_ntt_global_radix2.cuh:104-113). */
int stntt_set_coop(stntt_ctx *ctx, int mode);
int stntt_device_status(stntt_ctx *ctx);
/* Launch the staged kernel with no copy issued, so that its first wait runs
 * out after spin_limit polls; returns STNTT_ETIMEOUT when the kernel reported
 * it (the context stays usable). */
int stntt_selftest_tma_timeout(stntt_ctx *ctx, uint32_t spin_limit);

/* ---- polynomial multiplication (pwcNtt / pwc_convolution, ntt_cpu.cpp:167-193) */
/* d_out = cyclic convolution of d_a and d_b, length 2^log_n, i.e. the product
 * a*b mod (x^n - 1); equal to the plain product when deg a + deg b < n.
 * d_out may alias d_a or d_b. */
int stntt_polymul_u32(stntt_ctx *ctx, const uint32_t *d_a, const uint32_t *d_b, uint32_t *d_out, uint32_t log_n,
                      uint32_t p, uint32_t root, stntt_stream stream);
int stntt_polymul_gl64(stntt_ctx *ctx, const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_out, uint32_t log_n,
                       stntt_stream stream);
/* d_out[i] = d_a[i] * d_b[i] mod p (elemWiseMul, src/ntt/ntt_util.h:29-33). */
int stntt_pointwise_mul_u32(const uint32_t *d_a, const uint32_t *d_b, uint32_t *d_out, size_t count, uint32_t p,
                            stntt_stream stream);
int stntt_pointwise_mul_gl64(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_out, size_t count,
                             stntt_stream stream);

/* ---- serving loop ------------------------------------------------------------------ */
/* A request loop on one GPU (no counterpart in the reference; it composes
 * nttStockham and pwcNtt, src/ntt/ntt_cpu.cpp:46-90,167-174). A scheduler
 * thread admits requests in arrival order as soon as a stream slot is free and
 * the server's device arena can hold their operands, runs each on its own
 * stream (H2D, kernels, D2H) so requests overlap on the device, and records
 * host timestamps. Host buffers should be pinned and must stay valid until the
 * request completes. */
#define STNTT_REQ_NTT 0u
#define STNTT_REQ_POLYMUL 1u /* cyclic product of in_a and in_b, length 2^log_n */
typedef struct stntt_request {
    uint32_t kind, field, log_n, dir; /* dir: STNTT_REQ_NTT only */
    uint32_t p, root;                 /* STNTT_FIELD_U32 only */
    uint64_t id;                      /* echoed in the completion */
    const void *in_a, *in_b;          /* host operands (in_b: polymul) */
    void *out;                        /* host result, 2^log_n elements */
} stntt_request;
typedef struct stntt_completion {
    uint64_t id;
    int32_t status; /* STNTT_OK, or why the request failed */
    uint32_t reserved;
    double submit_s, start_s, done_s; /* stntt_clock_s() at submit, admission, completion */
} stntt_completion;
typedef struct stntt_server_config {
    uint32_t streams;      /* request slots (CUDA streams); 0 = 32 */
    uint32_t max_log_n;    /* largest request; per-slot workspaces are sized for it; 0 = 22 */
    uint64_t arena_bytes;  /* device memory for operands; 0 = a quarter of free HBM, at most 8 GiB */
    uint32_t prewarm_min_log_n, prewarm_max_log_n; /* build twiddle tables for this range at start */
} stntt_server_config;
typedef struct stntt_server_stats {
    uint64_t submitted, admitted, completed, failed, rejected;
    uint64_t peak_inflight, arena_bytes, peak_arena_used;
    /* scheduler-thread time: issuing admitted requests (copies, kernels,
     * events) and checking slots for completion, in nanoseconds */
    uint64_t issue_ns, poll_ns;
    /* stntt_server_run_trace only: the latest a request was handed to the
     * server after its arrival time (the load driver's own lag, counted in
     * the request's latency), and how many were more than 0.5 ms late */
    uint64_t trace_late_max_ns, trace_late_count;
} stntt_server_stats;
typedef struct stntt_server stntt_server;
double stntt_clock_s(void);
int stntt_server_create(stntt_ctx *ctx, const stntt_server_config *cfg, stntt_server **out);
int stntt_server_submit(stntt_server *sv, const stntt_request *req);
/* submit with an explicit arrival time (stntt_clock_s units) for latency accounting */
int stntt_server_submit_at(stntt_server *sv, const stntt_request *req, double t_submit);
int stntt_server_poll(stntt_server *sv, stntt_completion *out, size_t max, size_t *got);
int stntt_server_wait_idle(stntt_server *sv, double timeout_s);
int stntt_server_stats_get(stntt_server *sv, stntt_server_stats *out);
/* Native load driver: submits reqs[i] (whose id must be i) at arrival_s[i]
 * seconds after the start, waits for all, writes completion i to out[i]. */
int stntt_server_run_trace(stntt_server *sv, const stntt_request *reqs, const double *arrival_s, size_t n,
                           double timeout_s, stntt_completion *out);
int stntt_server_destroy(stntt_server *sv);

/* ---- allocation-free variant ------------------------------------------------------ */
/* No counterpart in the reference. For callers that cannot call cudaMalloc
 * (a memory pool that already owns HBM, a host runtime that manages device
 * memory itself, a loop that cannot take an allocation's synchronisation):
 * the same Goldilocks transform as stntt_ntt_gl64_oop, without a context and
 * without allocating. Its between-pass buffer and twiddle tables live in a
 * fixed array inside the library (8 MiB + 256 KiB per GPU, kept until exit),
 * so batch * 2^log_n must be <= 2^20 (else STNTT_EUNSUPPORTED). All calls
 * share that array: calls that overlap on the GPU race, so order them on one
 * stream. CUDA loads the library's device code on first use, so the first
 * call on a device may reserve the array and load the kernels: make that
 * first call (a warm-up) before a pool takes the rest of HBM and before
 * capturing a stream into a CUDA graph; if the array cannot be placed the
 * call returns STNTT_ENOMEM. d_in may equal d_out. */
int stntt_ntt_gl64_noalloc(const uint64_t *d_in, uint64_t *d_out, uint32_t log_n, uint32_t batch, int dir,
                           stntt_stream stream);

/* ---- integer roofline ---------------------------------------------------------- */
/* Goldilocks butterflies per second (add, sub and one product per butterfly)
 * that this GPU sustains on register-resident data, measured with the tile
 * kernel's own arithmetic and CUDA events: the integer roofline for the
 * transforms. Synchronous; about 10 ms. */
int stntt_measure_gl64_butterfly_rate(int device, double *butterflies_per_s);

/* ---- synthetic inputs ------------------------------------------------------------ */
/* Uniform residues in [0,p) from a counter-based splitmix64 stream:
 * element i, attempt a: z = mix64(seed + 0x9E3779B97F4A7C15 * (i + (a << 40) + 1));
 * u32 accepts (z >> 32) below the largest multiple of p and returns it mod p;
 * gl64 accepts z < p. */
int stntt_fill_uniform_u32(uint32_t *d_out, size_t count, uint64_t seed, uint32_t p, stntt_stream stream);
int stntt_fill_uniform_gl64(uint64_t *d_out, size_t count, uint64_t seed, stntt_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* STNTT_H */
