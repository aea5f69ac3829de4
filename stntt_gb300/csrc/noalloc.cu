// noalloc.cu -- a Goldilocks NTT entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs while a pre-reserved
// memory pool owns all of HBM, hosts that manage device memory themselves
// and forbid other allocators, and latency-critical loops that cannot afford
// the device-wide synchronisation an allocation may cause. For them,
// stntt_ntt_gl64_noalloc() runs the same tile kernels as stntt_ntt_gl64_oop()
// but keeps everything the transform needs beyond its input and output (the
// buffer between the two HBM passes and the twiddle tables) in the
// file-scope array below. It needs no context, calls no cudaMalloc/cudaFree
// and no allocating library routine.
//
// Limits and rules:
//   - batch * 2^log_n <= 2^20 elements (the array holds 8 MiB of data plus
//     256 KiB of twiddles; every GPU that loads the library keeps it until
//     the process exits). Larger sizes return STNTT_EUNSUPPORTED.
//   - All calls share the array and leave their data in it. Nothing in it
//     has to start at zero: each call regenerates its twiddles and overwrites
//     the data region before reading it. Calls whose work overlaps on the GPU
//     (different streams, or several host threads) race on the array; order
//     them on one stream or synchronise between them.
//   - Every call looks up the array's device address (cudaGetSymbolAddress)
//     with the caller's device current: a host-side lookup once the library's
//     device code is loaded, and correct again after a device reset, which
//     places the array at a new address. CUDA loads device code lazily, so
//     the first call on a device may load it and reserve the array and the
//     tile kernels' code at that moment: make that first call (a warm-up)
//     before a memory pool takes the rest of HBM and before capturing a
//     stream into a CUDA graph. If the array cannot be placed the call
//     returns STNTT_ENOMEM.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/stntt.h"
#include "internal.h"

namespace {

using namespace stntt;

constexpr uint32_t kMaxLogElems = 20;                  // batch * n <= 2^20
constexpr uint64_t kDataEntries = 1ull << kMaxLogElems;  // between-pass buffer, u64 elements
constexpr uint64_t kTableEntries = 1ull << 15;           // twiddle entries (8 bytes each)
constexpr uint64_t kGlP = 0xFFFFFFFF00000001ull;

static __device__ __align__(256) uint64_t g_noalloc_scratch[kDataEntries + kTableEntries];

// The device address of g_noalloc_scratch on the current device. In host
// code the array's name stands for a host-side shadow, never a device
// address; only this lookup gives the address kernels may use.
int scratch_address(uint64_t **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();  // clear the sticky-free error so later calls are not affected
        return e == cudaErrorMemoryAllocation ? STNTT_ENOMEM : STNTT_ECUDA;
    }
    *out = static_cast<uint64_t *>(p);
    return STNTT_OK;
}

uint32_t lg2(uint64_t v) {
    uint32_t l = 0;
    while ((1ull << l) < v)
        ++l;
    return l;
}

// Tile geometry for one Goldilocks pass (8-byte values: shared memory padded
// by one element per 16, column stride chosen so columns fall in different
// bank groups).
void shape(PassDesc &d, uint64_t col_limit) {
    const uint32_t L = 1u << d.logL;
    d.E = L < 16 ? L : (L >= 4096 ? 32 : 16);
    const uint32_t U = L / d.E;
    const uint32_t max_threads = d.E >= 32 ? 512 : 1024;
    uint64_t C = (d.mode == kModeRow && d.logN == d.logL) ? std::max<uint64_t>(1, 256 / U)
                                                           : std::min<uint64_t>(16, 16384 / L);
    C = std::min<uint64_t>({C, max_threads / U, col_limit, 64});
    C = std::max<uint64_t>(C, 1);
    d.logC = lg2(C);
    d.threads = (uint32_t)(C * U);
    const uint32_t banks = 16, base = L + (L >> 4);
    // odd stride from C = banks up: each phase reads one row of C columns
    const uint32_t want = d.tfast ? (U < banks ? U : 0) : (C < banks ? (uint32_t)(banks / C) : 1);
    d.cs = base + ((want + banks - base % banks) % banks);
    d.smem_bytes = (size_t)C * d.cs * 8;
}

}  // namespace

extern "C" int stntt_ntt_gl64_noalloc(const uint64_t *d_in, uint64_t *d_out, uint32_t log_n, uint32_t batch,
                                      int dir, stntt_stream stream) {
    if (dir != STNTT_FORWARD && dir != STNTT_INVERSE)
        return STNTT_EINVAL;
    if ((!d_in || !d_out) && batch)
        return STNTT_EINVAL;
    if (log_n > kMaxLogElems || ((uint64_t)batch << log_n) > kDataEntries)
        return STNTT_EUNSUPPORTED;  // beyond the fixed scratch: batch * 2^log_n must be <= 2^20
    if (batch == 0)
        return STNTT_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (log_n == 0) {
        if (d_in != d_out &&
            cudaMemcpyAsync(d_out, d_in, (size_t)batch * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return STNTT_ECUDA;
        return STNTT_OK;
    }
    uint64_t *scratch = nullptr;
    const int rc = scratch_address(&scratch);
    if (rc != STNTT_OK)
        return rc;
    uint64_t *data = scratch, *tables = scratch + kDataEntries;

    const uint64_t n = 1ull << log_n;
    uint64_t root = host_gl_pow(7, (kGlP - 1) >> log_n);
    if (dir == STNTT_INVERSE)
        root = host_gl_pow(root, kGlP - 2);
    const uint64_t ninv = dir == STNTT_INVERSE ? host_gl_pow(n, kGlP - 2) : 1;

    uint64_t off = 0;
    auto table = [&](uint64_t count, uint64_t base, uint64_t scale, uint64_t *o) {
        if (off + count > kTableEntries)
            return false;
        *o = off;
        if (launch_gen_powers(kFieldGL, tables + off, count, base, scale, 0, s) != cudaSuccess)
            return false;
        off += count;
        return true;
    };

    PassDesc passes[2];
    uint32_t K = log_n <= 13 ? 1 : 2;
    const uint32_t logs[2] = {K == 1 ? log_n : log_n / 2, log_n - log_n / 2};
    uint32_t done = 0;
    for (uint32_t i = 0; i < K; ++i) {
        PassDesc &d = passes[i];
        d.logL = logs[i];
        d.logN = log_n;
        const uint32_t L = 1u << d.logL;
        const uint64_t wL = host_gl_pow(root, n >> d.logL);
        if (!table(L, wL, 1, &d.tw_off))
            return STNTT_ECUDA;
        if (L >= 16) {
            const uint64_t w16 = host_gl_pow(wL, L / 16);
            for (int j = 0; j < 8; ++j)
                d.wR[j] = host_gl_pow(w16, j);
        } else {
            for (uint32_t j = 0; j < L / 2; ++j)
                d.wR[j * 16 / L] = host_gl_pow(wL, j);
        }
        d.scale = ninv;
        d.pow2 = dir == STNTT_INVERSE ? 2 : 1;  // the standard roots (see PassDesc::pow2)
        uint64_t col_limit;
        if (i + 1 < K) {
            d.mode = kModeCol;
            d.tfast = 0;
            d.logM = log_n - done;
            d.logS = d.logM - d.logL;
            d.h = (d.logM + 1) / 2;
            const uint64_t wM = host_gl_pow(root, n >> d.logM);
            if (!table(1ull << d.h, wM, 1, &d.lo_off) ||
                !table(1ull << (d.logM - d.h), host_gl_pow(wM, 1ull << d.h), i == 0 ? ninv : 1, &d.hi_off))
                return STNTT_ECUDA;
            col_limit = 1ull << d.logS;
        } else {
            d.mode = kModeRow;
            d.tfast = K == 1 ? 1 : 0;
            d.do_scale = (K == 1 && dir == STNTT_INVERSE) ? 1 : 0;
            d.logN1 = K == 2 ? logs[0] : 0;
            d.logN2 = 0;
            col_limit = 1ull << 20;
        }
        shape(d, col_limit);
        done += d.logL;
    }
    const void *src = d_in;
    for (uint32_t i = 0; i < K; ++i) {
        void *dst = (i + 1 == K) ? static_cast<void *>(d_out) : static_cast<void *>(data);
        if (launch_tile(kFieldGL, passes[i], 0, tables, src, dst, batch, s) != cudaSuccess)
            return STNTT_ECUDA;
        src = dst;
    }
    return STNTT_OK;
}
