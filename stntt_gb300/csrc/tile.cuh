// tile.cuh -- the NTT tile kernel: C independent DFTs of length L per CTA.
//
// One kernel covers every HBM pass of the transform:
//   ROW pass: C rows, each contiguous in memory, written to a strided
//     (digit-reversed) position. With n == L this is the whole transform
//     of small sizes (the reference's stNttRadix2 / stNttRadix2Adaptive,
//     src/cuda/ntt/implementations/st_ntt_radix2*.cuh); with n > L it is the
//     last four-step pass.
//   COL pass: C adjacent columns at stride S, followed by the four-step
//     twiddle w_M^(col*k) (and n^-1 for the first inverse pass).
// Together they replace the reference's log2(n)-10 one-stage-per-launch
// passes (stNttGlobalRadix2_first/_rest, st_ntt_global_radix2.cuh:8-117) and
// the in-block stNttLocalRadix2 (st_ntt_local_radix2.cuh:5-110) with 1-3
// HBM passes.
//
// Inside a tile: radix-16 Stockham DIT steps (one leading radix-2/4/8 step
// when log2 L is not a multiple of 4), or radix-8 steps for the builds with 8
// elements per thread (tile_steps_l). A step reads R values per item into
// registers, applies w_(R p)^(r k), runs an R-point DFT as a radix-2 network
// in registers, and writes to shared memory in Stockham order. The first
// step reads HBM directly and the last writes HBM directly, so each element
// crosses HBM once per pass. Shared memory is padded (one element per 32
// for 4-byte, per 16 for 8-byte values) so the Stockham patterns avoid bank
// conflicts.
#pragma once
#include <cstdint>

#include "fields.cuh"
#include "internal.h"

namespace stntt {

// Programmatic dependent launch (no-ops for a launch without the
// programmatic-serialization attribute): a kernel waits until the previous
// kernel's writes are visible before it touches global memory, and lets the
// next kernel start launching once it reaches its last step (so that the next
// kernel's CTAs take SM slots only near the end of this one).
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class F>
struct TileArgs {
    using T = typename F::T;
    using TW = typename F::TW;
    const T *in;
    T *out;
    const TW *twL;     // w_L^e, e < L
    const TW *tw4_lo;  // COL: w_M^e, e < 2^h
    const TW *tw4_hi;  // COL: s * w_M^(e * 2^h), e < M / 2^h  (s = n^-1 on the first inverse pass)
    const TW *tw4_full;  // COL, optional: lo * hi for every (pos, col), at pos * S + col
    TW wR[8];          // w_16^j (for L < 16: entry j*16/L holds w_L^j)
    TW scale;          // ROW with do_scale: n^-1
    uint32_t p;
    uint32_t logL, logC, mode, do_scale, tfast, h;
    uint32_t logN;          // elements per transform
    uint32_t logM, logS;    // COL: sub-problem size, column stride
    uint32_t logN1, logN2;  // ROW: rows r map to input row ((r mod n1) * n2 + r / n1)
    uint32_t cs;            // shared-memory column stride, elements
    uint64_t total;         // columns (COL) or rows (ROW) over the whole batch
    // Optional per-transform base pointers (batched jobs): transform b reads
    // from in_ptrs[b] and writes to out_ptrs[b] instead of in/out + b*n.
    const unsigned long long *in_ptrs;
    const unsigned long long *out_ptrs;
    // Optional second input (pointwise product fused into the first step):
    // the pass transforms in[j] * in2[j] (same layout as in).
    const T *in2;
    // COL, 32-bit field, vector-lines build only: the full four-step table in
    // Montgomery form (4 bytes per entry, w * 2^32 mod p, at pos * S + col)
    // and pinv = -p^-1 mod 2^32.
    const uint32_t *tw4_mont;
    uint32_t pinv;
    // Goldilocks: PassDesc::pow2 (1 forward root, 2 inverse root, 0 other);
    // the batched kernel picks the direction-specialised field type by it.
    uint32_t pow2;
    // Batched launch: 2 when this pass's items run the vector-lines steps
    // (two lines per thread, 16-byte accesses; every job pointer 16-byte
    // aligned), else 0.
    uint32_t vecl;
};

template <class F>
struct Pad;
template <>
struct Pad<FieldU32> {
    static constexpr uint32_t PS = 5;
    static __device__ __forceinline__ uint32_t at(uint32_t i) { return i + (i >> 5); }
};
template <>
struct Pad<FieldU32L> {
    static constexpr uint32_t PS = 5;
    static __device__ __forceinline__ uint32_t at(uint32_t i) { return i + (i >> 5); }
};
template <>
struct Pad<FieldGL> {
    static constexpr uint32_t PS = 4;
    static __device__ __forceinline__ uint32_t at(uint32_t i) { return i + (i >> 4); }
};
template <int DIR>
struct Pad<FieldGLPow2<DIR>> : Pad<FieldGL> {};

template <int LOGR>
__host__ __device__ constexpr int bit_reverse(int r) {
    int y = 0;
    for (int i = 0; i < LOGR; ++i)
        y |= ((r >> i) & 1) << (LOGR - 1 - i);
    return y;
}

// R-point DFT with root w_R, as a radix-2 DIF network: natural order in,
// bit-reversed order out. Span-2h stages use w_(2h)^j = w_16^(j*16/(2h)).
template <class F, int R>
__device__ __forceinline__ void dft_reg(const F &f, typename F::T *x, const typename F::TW *w16) {
#pragma unroll
    for (int h = R / 2; h >= 1; h >>= 1) {
#pragma unroll
        for (int base = 0; base < R; base += 2 * h) {
#pragma unroll
            for (int j = 0; j < h; ++j) {
                const typename F::T a = x[base + j], b = x[base + j + h];
                if constexpr (IsPow2Field<F>::value) {
                    // w_16^q = +-2^e: the sign by the order of the subtraction
                    const int q = j * (16 / (2 * h)), e = F::w16_exp(q);
                    x[base + j] = f.add(a, b);
                    x[base + j + h] = j == 0 ? f.sub(a, b) : f.mul_pow2(e >= 96 ? f.sub(b, a) : f.sub(a, b), e % 96);
                } else {
                    const typename F::T d = j == 0 ? f.sub(a, b) : f.sub_lazy(a, b);
                    x[base + j] = f.add(a, b);
                    x[base + j + h] = j == 0 ? d : f.mul_tw(d, w16[j * (16 / (2 * h))]);
                }
            }
        }
    }
}

template <class T>
struct Geo {
    const T *src;   // element j of this column/row
    const T *src2;  // second input for the fused pointwise product, or null
    T *dst;        // element k of the output
    uint32_t istride, ostride;  // element j at src[j * istride], k at dst[k * ostride] (< 2^32)
    uint32_t col;             // COL: column index within the sub-problem (< 2^28)
    bool valid;  // false for the padding rows of a partial last CTA
};

// The four-step twiddle w_M^(col * pos) of a column pass's output pos: one
// entry of the full table (FULL4) or the product of two table entries.
template <class F, bool FULL4>
__device__ __forceinline__ typename F::T four_step(const TileArgs<F> &a, const F &f, const Geo<typename F::T> &g,
                                                   uint32_t pos, typename F::T v) {
    if constexpr (FULL4) {
        return f.mul_tw(v, __ldg(&a.tw4_full[(uint64_t)pos * g.ostride + g.col]));
    } else {
        const uint64_t e = (uint64_t)g.col * pos;
        const uint32_t lo = (uint32_t)(e & ((1ull << a.h) - 1));
        const uint32_t hi = (uint32_t)(e >> a.h);
        return f.mul_tw(f.mul_tw(v, __ldg(&a.tw4_lo[lo])), __ldg(&a.tw4_hi[hi]));
    }
}

// Output k = pos of a tile's last step: the four-step twiddle (COL) or n^-1
// (ROW with do_scale), then the canonical value to HBM.
template <class F, bool FULL4 = false>
__device__ __forceinline__ void store_last(const TileArgs<F> &a, const F &f, const Geo<typename F::T> &g,
                                           uint32_t pos, typename F::T v) {
    if (a.mode == kModeCol)
        v = four_step<F, FULL4>(a, f, g, pos, v);
    else if (a.do_scale)
        v = f.mul_tw(v, a.scale);
    v = f.canon(v);
    if (g.valid)
        g.dst[(uint64_t)pos * g.ostride] = v;
}

template <class F, int E, int LOGR, bool first, bool last, bool in2 = false>
__device__ __forceinline__ void tile_step(const TileArgs<F> &a, const F &f, typename F::T (&x)[E],
                                          typename F::T *sm, uint32_t c, uint32_t u, uint32_t logp,
                                          const Geo<typename F::T> &g) {
    using T = typename F::T;
    constexpr int R = 1 << LOGR, ITEMS = E / R;
    const uint32_t L = 1u << a.logL, U = L / E, T_ = L >> LOGR;
    if constexpr (last)
        pdl_trigger();
    const uint32_t pm = (1u << logp) - 1;
    T *col_sm = sm + c * a.cs;

    // ---- read R inputs per item: idx = t + r * L/R
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        const uint32_t t = u + m * U;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t idx = t + r * T_;
            if constexpr (first) {
                x[m * R + r] = g.valid ? g.src[(uint64_t)idx * g.istride] : T(0);
                if constexpr (in2) {
                    if (g.valid)
                        x[m * R + r] = f.mul(x[m * R + r], g.src2[(uint64_t)idx * g.istride]);
                }
            }
            else
                x[m * R + r] = col_sm[Pad<F>::at(idx)];
        }
    }
    // ---- twiddle w_(R p)^(r k) = w_L^(r k L/(R p)), k = t mod p; then R-point DFT
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        const uint32_t t = u + m * U;
        if constexpr (!first) {
            const uint32_t k = t & pm;
            const uint32_t sh = a.logL - LOGR - logp;
#pragma unroll
            for (int r = 1; r < R; ++r)
                x[m * R + r] = f.mul_tw(x[m * R + r], __ldg(&a.twL[(r * k) << sh]));
        }
        dft_reg<F, R>(f, &x[m * R], a.wR);
    }
    if constexpr (!first && !last)
        __syncthreads();  // every read of this step precedes any write
    // ---- write output r of item t to (t - k) R + k + r p
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        const uint32_t t = u + m * U;
        const uint32_t k = t & pm;
        const uint32_t base = ((t - k) << LOGR) + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t pos = base + ((uint32_t)r << logp);
            T v = x[m * R + bit_reverse<LOGR>(r)];
            if constexpr (last) {
                store_last(a, f, g, pos, v);
            } else {
                col_sm[Pad<F>::at(pos)] = v;
            }
        }
    }
    if constexpr (!last)
        __syncthreads();
}

// The first step of a tile (the optional radix-2/4/8 step, else radix 16).
// Returns true when it was also the last step.
template <class F, int E, int TAIL, bool IN2>
__device__ __forceinline__ bool first_step(const TileArgs<F> &a, const F &f, typename F::T (&x)[E],
                                           typename F::T *sm, uint32_t c, uint32_t u, const Geo<typename F::T> &g,
                                           uint32_t &logp) {
    const int n16 = (int)(a.logL >> 2);
    if constexpr (TAIL > 0) {
        if (n16 == 0) {
            tile_step<F, E, TAIL, true, true, IN2>(a, f, x, sm, c, u, 0, g);
            return true;
        }
        tile_step<F, E, TAIL, true, false, IN2>(a, f, x, sm, c, u, 0, g);
        logp = TAIL;
    } else {
        if (n16 == 1) {
            tile_step<F, E, 4, true, true, IN2>(a, f, x, sm, c, u, 0, g);
            return true;
        }
        tile_step<F, E, 4, true, false, IN2>(a, f, x, sm, c, u, 0, g);
        logp = 4;
    }
    return false;
}

// Which column (COL) or row (ROW) thread threadIdx.x works on, its index u
// within it, and the HBM addresses of its first and last step.
template <class F, int E>
__device__ __forceinline__ Geo<typename F::T> tile_geo(const TileArgs<F> &a, uint64_t blk, uint32_t &c,
                                                       uint32_t &u) {
    using T = typename F::T;
    const uint32_t C = 1u << a.logC;
    constexpr uint32_t logE = E >= 32 ? 5 : E >= 16 ? 4 : E >= 8 ? 3 : E >= 4 ? 2 : 1;
    const uint32_t logU = a.logL - logE;  // log2(L / E): threads per column
    if (a.tfast) {
        u = threadIdx.x & ((1u << logU) - 1);
        c = threadIdx.x >> logU;
    } else {
        c = threadIdx.x & (C - 1);
        u = threadIdx.x >> a.logC;
    }
    // global column / row index over the whole batch
    const uint64_t gi = (blk << a.logC) + c;
    const uint32_t logPer = a.logN - a.logL;  // columns (rows) per transform
    const uint64_t b = gi >> logPer;
    const uint64_t rem = gi & ((1ull << logPer) - 1);
    Geo<T> g;
    g.valid = gi < a.total;
    const T *ibase = a.in + (b << a.logN);
    T *obase = a.out + (b << a.logN);
    if (a.in_ptrs && g.valid) {
        ibase = reinterpret_cast<const T *>(a.in_ptrs[b]);
        obase = reinterpret_cast<T *>(a.out_ptrs[b]);
    }
    const T *ibase2 = a.in2 ? a.in2 + (b << a.logN) : nullptr;
    g.src2 = nullptr;
    if (a.mode == kModeCol) {
        const uint64_t q = rem >> a.logS;
        g.col = (uint32_t)(rem & ((1ull << a.logS) - 1));
        g.src = ibase + (q << a.logM) + g.col;
        if (ibase2)
            g.src2 = ibase2 + (q << a.logM) + g.col;
        g.dst = obase + (q << a.logM) + g.col;
        g.istride = g.ostride = 1u << a.logS;
    } else {
        const uint64_t inrow = ((rem & ((1ull << a.logN1) - 1)) << a.logN2) + (rem >> a.logN1);
        g.col = 0;
        g.src = ibase + (inrow << a.logL);
        if (ibase2)
            g.src2 = ibase2 + (inrow << a.logL);
        g.istride = 1;
        g.dst = obase + rem;
        g.ostride = 1u << logPer;
    }
    return g;
}

// One CTA's worth of work: C columns (COL) or rows (ROW) with global index
// blk * C + c over the batch. Used by tile_kernel (blk = blockIdx.x) and by
// the persistent batched kernel (blk from its work list).
template <class F, int E, int TAIL, bool IN2 = false>
__device__ __forceinline__ void tile_run(const TileArgs<F> &a, uint64_t blk, typename F::T *sm) {
    using T = typename F::T;
    F f;
    f.p = a.p;

    uint32_t c, u;
    const Geo<T> g = tile_geo<F, E>(a, blk, c, u);

    T x[E];
    const int n16 = (int)(a.logL >> 2);  // radix-16 steps after the optional leading step
    uint32_t logp = 0;
    // the first step (with the fused pointwise product when IN2)
    if (first_step<F, E, TAIL, IN2>(a, f, x, sm, c, u, g, logp))
        return;
    if constexpr (E >= 16) {
        const int mid = n16 - (TAIL > 0 ? 1 : 2);  // radix-16 steps between the first and the last
        for (int s = 0; s < mid; ++s) {
            tile_step<F, E, 4, false, false>(a, f, x, sm, c, u, logp, g);
            logp += 4;
        }
        tile_step<F, E, 4, false, true>(a, f, x, sm, c, u, logp, g);
    }
}


template <class F, int E, int TAIL, bool IN2 = false>
__global__ void __launch_bounds__(E >= 32 ? 512 : 1024) tile_kernel(const TileArgs<F> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    tile_run<F, E, TAIL, IN2>(a, blockIdx.x, reinterpret_cast<typename F::T *>(smem_raw));
}

// Where a tile's first step reads and its last step writes: HBM through the
// tile geometry (the four-step twiddle or scale applied on the way out).
template <class F, bool FULL4>
struct GlobalIO {
    using T = typename F::T;
    Geo<T> g;
    __device__ __forceinline__ T load(uint32_t idx) const { return g.valid ? g.src[(uint64_t)idx * g.istride] : T(0); }
    __device__ __forceinline__ void store(const TileArgs<F> &a, const F &f, uint32_t pos, T v) const {
        store_last<F, FULL4>(a, f, g, pos, v);
    }
};

// ---- Tile length fixed at compile time -----------------------------------
// The same Stockham steps with L = 2^LOGL a template parameter and 16
// elements per thread: each step's stride, twiddle shift and output spacing
// are constants, so shared-memory indices are a per-thread padded base plus
// an immediate. The padding never separates an access from its base:
// Pad(b + d) = Pad(b) + d + (d >> PS) for every read (b = u, d = m U + r L/R)
// and every write (b = the item's output base, d = r p) of these steps.
template <class F, int E, int LOGL, int LOGR, int LOGP, bool first, bool last, class IO>
__device__ __forceinline__ void tile_step_l(const TileArgs<F> &a, const F &f, typename F::T (&x)[E],
                                            typename F::T *col_sm, uint32_t u, const IO &io) {
    using T = typename F::T;
    constexpr int R = 1 << LOGR, ITEMS = E / R;
    constexpr uint32_t PS = Pad<F>::PS, U = (1u << LOGL) / E, TS = (1u << LOGL) >> LOGR, P = 1u << LOGP;
    static_assert(LOGR + LOGP <= LOGL, "step beyond the tile");
    if constexpr (last)
        pdl_trigger();
    // ---- read R inputs per item: idx = u + m U + r L/R
    const uint32_t pu = Pad<F>::at(u);
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t d = m * U + r * TS;
            if constexpr (first)
                x[m * R + r] = io.load(u + d);
            else
                x[m * R + r] = col_sm[pu + d + (d >> PS)];
        }
    }
    // ---- twiddle w_(R p)^(r k), k = t mod p, then the R-point DFT
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        if constexpr (!first) {
            const uint32_t k = (u + m * U) & (P - 1);
#pragma unroll
            for (int r = 1; r < R; ++r)
                x[m * R + r] = f.mul_tw(x[m * R + r], __ldg(&a.twL[(r * k) << (LOGL - LOGR - LOGP)]));
        }
        dft_reg<F, R>(f, &x[m * R], a.wR);
    }
    if constexpr (!first && !last)
        __syncthreads();  // every read of this step precedes any write
    // ---- write output r of item t to (t - k) R + k + r p
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        const uint32_t t = u + m * U;
        const uint32_t k = t & (P - 1);
        const uint32_t base = ((t - k) << LOGR) + k;
        const uint32_t pb = Pad<F>::at(base);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t d = (uint32_t)r << LOGP;
            const T v = x[m * R + bit_reverse<LOGR>(r)];
            if constexpr (last)
                io.store(a, f, base + d, v);
            else
                col_sm[pb + d + (d >> PS)] = v;
        }
    }
    if constexpr (!last)
        __syncthreads();
}

// Steps S.. of a 2^LOGL tile with E elements per thread: one leading
// radix-2^(LOGL mod log2 E) step when needed, then radix-E steps (E = 16, or
// 8 for twice the threads on small transforms). The padding identity above
// holds for both (checked exhaustively for every L up to 2^13).
template <class F, int E, int LOGL, int S, class IO>
__device__ __forceinline__ void tile_steps_l(const TileArgs<F> &a, const F &f, typename F::T (&x)[E],
                                             typename F::T *col_sm, uint32_t u, const IO &io) {
    static_assert(E == 8 || E == 16, "radix-8 or radix-16 steps");
    constexpr int LE = E == 8 ? 3 : 4;  // log2 of the radix of the full steps
    constexpr int TAIL = LOGL % LE;
    constexpr int NS = LOGL / LE + (TAIL > 0 ? 1 : 0);
    if constexpr (S < NS) {
        constexpr int LOGR = (S == 0 && TAIL > 0) ? TAIL : LE;
        constexpr int LOGP = S == 0 ? 0 : (TAIL > 0 ? TAIL + LE * (S - 1) : LE * S);
        tile_step_l<F, E, LOGL, LOGR, LOGP, S == 0, S == NS - 1, IO>(a, f, x, col_sm, u, io);
        tile_steps_l<F, E, LOGL, S + 1, IO>(a, f, x, col_sm, u, io);
    }
}

// One CTA's worth of work with the tile length compiled in (the counterpart
// of tile_run for 16 elements per thread).
template <class F, int LOGL, bool FULL4 = false, int E = 16>
__device__ __forceinline__ void tile_run_l(const TileArgs<F> &a, uint64_t blk, typename F::T *sm) {
    static_assert(LOGL >= (E == 8 ? 3 : 4), "a tile holds at least one thread's elements");
    using T = typename F::T;
    F f;
    f.p = a.p;
    uint32_t c, u;
    const Geo<T> g = tile_geo<F, E>(a, blk, c, u);
    T x[E];
    tile_steps_l<F, E, LOGL, 0, GlobalIO<F, FULL4>>(a, f, x, sm + c * a.cs, u, GlobalIO<F, FULL4>{g});
}

// MINB > 1: a build for CTAs of at most 256 threads with MINB of them resident
// per SM (registers capped at 65536 / (256 MINB) per thread). E: elements per
// thread (16, or 8 for twice the threads on small transforms).
template <class F, int LOGL, bool FULL4 = false, int MINB = 1, int E = 16>
__global__ void __launch_bounds__(MINB > 1 ? 256 : 1024, MINB) tile_kernel_l(const TileArgs<F> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    tile_run_l<F, LOGL, FULL4, E>(a, blockIdx.x, reinterpret_cast<typename F::T *>(smem_raw));
}

}  // namespace stntt
