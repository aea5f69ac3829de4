// tile_v.cuh -- the tile kernel with V adjacent lines per thread and 16-byte
// vector accesses (HBM and shared memory), for the passes of large
// transforms.
//
// The passes are those of tile.cuh (COL: C adjacent columns of a four-step
// sub-problem, four-step twiddle on the way out; ROW: C adjacent rows, written
// to their digit-reversed positions), and the arithmetic is the same radix-16
// Stockham DIT steps in registers. What changes is the thread layout:
//   - a thread owns V lines side by side (4 four-byte or 2 eight-byte values,
//     16 bytes) and E points of each (16, or 8 for half the registers and
//     more resident warps); its V independent E-point DFTs share one set of
//     step-twiddle loads and index arithmetic;
//   - a column pass loads and stores 16 bytes per access (V adjacent columns
//     of one row); a row pass stores 16 bytes per access (V adjacent rows at
//     one output position) and loads V scalars;
//   - shared memory holds the tile point-major, [point][C lines]: each access
//     moves one thread's 16 bytes; with 8 line groups the 8 threads of a
//     quarter-warp phase cover one contiguous 128-byte row, so no padding is
//     needed for any Stockham stride; with 4 line groups some strided writes
//     meet two-way conflicts, and with 2 (the narrowest wide tiles) a 16-byte
//     pad after every 128 bytes of points keeps strided writes apart;
//   - the grid covers the lines exactly (the host only picks shapes where C
//     divides the lines of a sub-problem), so no access is predicated.
// Replaces, like tile.cuh, the reference's one-stage-per-launch global passes
// (stNttGlobalRadix2_first/_rest, st_ntt_global_radix2.cuh:8-117), whose
// loads and stores are one 4-byte element per access (:60-75, :95-100).
#pragma once
#include <cstdint>

#include "tile.cuh"

namespace stntt {

// 16 bytes of V elements: load / store between memory and V registers.
template <class T, int V>
__device__ __forceinline__ void v16_load(T (&x)[V], const T *p) {
    if constexpr (sizeof(T) == 4) {
        static_assert(V == 4, "16 bytes of 4-byte values");
        const uint4 q = *reinterpret_cast<const uint4 *>(p);
        x[0] = q.x, x[1] = q.y, x[2] = q.z, x[3] = q.w;
    } else {
        static_assert(V == 2, "16 bytes of 8-byte values");
        const ulonglong2 q = *reinterpret_cast<const ulonglong2 *>(p);
        x[0] = q.x, x[1] = q.y;
    }
}
template <class T, int V>
__device__ __forceinline__ void v16_store(T *p, const T (&x)[V]) {
    if constexpr (sizeof(T) == 4)
        *reinterpret_cast<uint4 *>(p) = make_uint4(x[0], x[1], x[2], x[3]);
    else
        *reinterpret_cast<ulonglong2 *>(p) = make_ulonglong2(x[0], x[1]);
}
// read-only global variant (through the non-coherent path)
template <class T, int V>
__device__ __forceinline__ void v16_ldg(T (&x)[V], const T *p) {
    if constexpr (sizeof(T) == 4) {
        const uint4 q = __ldg(reinterpret_cast<const uint4 *>(p));
        x[0] = q.x, x[1] = q.y, x[2] = q.z, x[3] = q.w;
    } else {
        const ulonglong2 q = __ldg(reinterpret_cast<const ulonglong2 *>(p));
        x[0] = q.x, x[1] = q.y;
    }
}

// V twiddle entries at p (consecutive, 16-byte aligned): u32 Shoup pairs are
// 8 bytes each (two 16-byte loads for V = 4), Goldilocks entries 8 bytes.
template <class F, int V>
__device__ __forceinline__ void tw_load_v(typename F::TW (&w)[V], const typename F::TW *p) {
    static_assert(sizeof(typename F::TW) == 8, "8-byte twiddle entries");
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
    for (int i = 0; i < V / 2; ++i) {
        const uint4 a = __ldg(q + i);
        const unsigned long long lo = ((unsigned long long)a.y << 32) | a.x;
        const unsigned long long hi = ((unsigned long long)a.w << 32) | a.z;
        memcpy(&w[2 * i], &lo, 8);
        memcpy(&w[2 * i + 1], &hi, 8);
    }
}

// Where a thread's lines start in HBM. Offsets from these pointers (idx *
// istride, pos * ostride + col0) stay below the points of one sub-problem or
// transform (at most 2^32), so 32-bit products are exact. The column loads
// and the Montgomery-table loads use them: with 64-bit products there, the
// 32-bit column kernels at 64 registers per thread spilled 60 to 140 bytes per
// thread (ptxas -v), with 32-bit ones the full-table builds spill nothing.
// The stores and the 8-byte table keep 64-bit products, which spilled least
// over all instantiations.
template <class T, int V>
struct VGeo {
    const T *src[V];   // COL: src[0] = element 0 of the thread's first column; ROW: row v's element 0
    T *dst;            // COL: element 0 of the first column; ROW: output slot of the first row
    uint32_t istride;  // COL: column stride (elements)
    uint32_t ostride;  // COL: column stride; ROW: n / L (the digit-reversed output spacing)
    uint32_t col0;     // COL: the thread's first column within its sub-problem
};

// FULL4: 0 two-level four-step lookup, 1 full table of twiddle entries,
// 2 full table of 4-byte Montgomery entries (32-bit field). BIN: the values
// arrive below BIN p (lazy 32-bit field; a four-step product leaves 2p).
template <class F, int V, bool COL, int FULL4, int BIN = 2>
__device__ __forceinline__ void vstore_last(const TileArgs<F> &a, const F &f, const VGeo<typename F::T, V> &geo,
                                            uint32_t pos, typename F::T (&v)[V]) {
    using TW = typename F::TW;
    if constexpr (COL) {
        if constexpr (FULL4 == 2) {
            static_assert(V == 4, "Montgomery tables serve the 32-bit field");
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(a.tw4_mont + (pos * geo.ostride + geo.col0)));
            v[0] = f.mul_mont(v[0], w.x, a.pinv);
            v[1] = f.mul_mont(v[1], w.y, a.pinv);
            v[2] = f.mul_mont(v[2], w.z, a.pinv);
            v[3] = f.mul_mont(v[3], w.w, a.pinv);
        } else if constexpr (FULL4 == 1) {
            TW w[V];
            tw_load_v<F, V>(w, a.tw4_full + (uint64_t)pos * geo.ostride + geo.col0);
#pragma unroll
            for (int i = 0; i < V; ++i)
                v[i] = f.mul_tw(v[i], w[i]);
        } else {
#pragma unroll
            for (int i = 0; i < V; ++i) {
                const uint32_t e = (geo.col0 + i) * pos;  // col * pos < M <= 2^32
                const uint32_t lo = e & ((1u << a.h) - 1u);
                const uint32_t hi = e >> a.h;
                v[i] = f.mul_tw(f.mul_tw(v[i], __ldg(&a.tw4_lo[lo])), __ldg(&a.tw4_hi[hi]));
            }
        }
    }
#pragma unroll
    for (int i = 0; i < V; ++i) {
        if constexpr (IsLazyBound<F>::value && !COL && BIN > 2)
            v[i] = f.template canon_b<BIN>(v[i]);
        else
            v[i] = f.canon(v[i]);
    }
    v16_store<typename F::T, V>(geo.dst + (uint64_t)pos * geo.ostride, v);
}

// Element offset of a point's C lines in the shared-memory tile. With 8 line
// groups (128 bytes per point) points are packed. With fewer, a quarter-warp
// phase (8 threads x 16 bytes) spans 8 / 2^LOGG points, and Stockham writes
// of points R apart land on the same banks. With 4 groups that is a two-way
// conflict on some writes (about 1% of a Goldilocks pass's instructions); a
// pad costs more index arithmetic than it saves there (Goldilocks 2^24
// forward + inverse 0.626 ms unpadded, 0.639 ms padded), so points stay
// packed. With 1 or 2 groups (the wide tiles of two-pass plans) it would be
// four- to eight-way: one 16-byte pad after every 8 / 2^LOGG points shifts
// consecutive 128-byte rows by a bank quarter (the plain build's padding
// scheme, at 16-byte granularity).
template <int V, int LOGG>
__device__ __forceinline__ constexpr uint32_t vpoint(uint32_t point) {
    constexpr uint32_t C = V << LOGG, PB = LOGG < 2 ? 3 - LOGG : 0;
    return PB ? point * C + (point >> PB) * V : point * C;
}

// ---- The R-point DIF network of dft_reg with bounds tracked at compile time
// (FieldU32L, p < 2^29). Every value is below B p for a known B <= 8, so a sum
// is one add (a + b < 8p), a difference one add (a - b + K p, K >= the bound
// of b), and a value is halved (red: one conditional subtraction) only where
// a butterfly would otherwise pass 8p; twiddled differences leave the Shoup
// product in [0, 2p). dft_reg keeps every sum and untwiddled difference in
// [0, 2p) (three operations each). Operation counts per 16-point DFT whose
// point 0 is below 8p and the others below 2p (later steps): 149 against
// 209; all inputs canonical (first step): 131. Outputs stay below LzPlan::bout
// p (at most 8), canonicalised once before the HBM store.
template <int R>
struct LzPlan {
    int ra[4][8], rb[4][8];  // per level and butterfly: halve a / b first (K, or 0)
    int kd[4][8];            // K of the difference a - b + K p
    int bout;                // bound of every output
};

__host__ __device__ constexpr int lz_pow2_at_least(int b) {
    int k = 1;
    while (k < b)
        k *= 2;
    return k;
}

// b0: bound of point 0 (not twiddled by the step), br: of the others.
template <int R>
__host__ __device__ constexpr LzPlan<R> lz_plan(int b0, int br) {
    LzPlan<R> P{};
    int B[16] = {};
    for (int i = 0; i < R; ++i)
        B[i] = i == 0 ? b0 : br;
    int l = 0;
    for (int h = R / 2; h >= 1; h /= 2, ++l) {
        int q = 0;
        for (int base = 0; base < R; base += 2 * h) {
            for (int j = 0; j < h; ++j, ++q) {
                const int a = base + j, b = a + h;
                // halve the larger input (to below K p, 2K >= its bound) until
                // the sum and the difference stay below 8p
                while (B[a] + B[b] > 8 || B[a] + lz_pow2_at_least(B[b]) > 8) {
                    const int x = B[a] >= B[b] ? a : b;
                    const int k = lz_pow2_at_least(B[x]) / 2;
                    int &slot = x == a ? P.ra[l][q] : P.rb[l][q];
                    if (slot != 0 || k == 0)
                        return LzPlan<R>{};  // bout 0: no plan (one halving per input)
                    slot = k;
                    B[x] = k;
                }
                P.kd[l][q] = lz_pow2_at_least(B[b]);
                const int s = B[a] + B[b];
                B[b] = j == 0 ? B[a] + P.kd[l][q] : 2;
                B[a] = s;
            }
        }
    }
    P.bout = 1;
    for (int i = 0; i < R; ++i)
        P.bout = B[i] > P.bout ? B[i] : P.bout;
    return P;
}

template <int R>
__host__ __device__ constexpr int lz_levels() {
    return R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
}

// Level L, butterfly Q of the network (same order and twiddles as dft_reg).
template <class F, int R, int B0, int BR, int L = 0, int Q = 0>
__device__ __forceinline__ void dft_lazy(const F &f, typename F::T *x, const typename F::TW *w16) {
    static_assert(IsLazyBound<F>::value, "bound-tracked DFT of the lazy 32-bit field");
    if constexpr (L < lz_levels<R>()) {
        constexpr LzPlan<R> P = lz_plan<R>(B0, BR);
        static_assert(P.bout >= 1 && P.bout <= 8, "values stay below 8p");
        constexpr int h = (R / 2) >> L, j = Q % h, a = (Q / h) * 2 * h + j, b = a + h;
        if constexpr (P.ra[L][Q] != 0)
            x[a] = f.red(x[a], P.ra[L][Q]);
        if constexpr (P.rb[L][Q] != 0)
            x[b] = f.red(x[b], P.rb[L][Q]);
        const uint32_t d = x[a] - x[b] + (uint32_t)P.kd[L][Q] * f.p;
        x[a] = x[a] + x[b];
        if constexpr (j == 0)
            x[b] = d;
        else
            x[b] = f.mul_tw(d, w16[j * (16 / (2 * h))]);
        if constexpr (Q + 1 < R / 2)
            dft_lazy<F, R, B0, BR, L, Q + 1>(f, x, w16);
        else
            dft_lazy<F, R, B0, BR, L + 1, 0>(f, x, w16);
    }
}

// Bounds entering a vector-lines step's DFTs: the first reads canonical
// values from HBM; later ones read point 0 as the previous step left it
// (below 8p) and the others after a Shoup product (below 2p).
template <bool first>
struct LzIn {
    static constexpr int b0 = first ? 1 : 8, br = first ? 1 : 2;
};

// One radix-2^LOGR Stockham step over the tile (see tile_step_l): read R
// points per item (HBM on the first step, else shared memory), twiddle,
// R-point DFT per line, write R points (shared memory, or HBM on the last).
template <class F, int V, int E, int LOGL, int LOGG, int LOGR, int LOGP, bool first, bool last, bool COL, int FULL4>
__device__ __forceinline__ void vstep(const TileArgs<F> &a, const F &f, typename F::T (&x)[V][E],
                                      typename F::T *sm_g, uint32_t u, const VGeo<typename F::T, V> &geo) {
    using T = typename F::T;
    constexpr int R = 1 << LOGR, ITEMS = E / R;
    constexpr uint32_t U = (1u << LOGL) / E, TS = (1u << LOGL) >> LOGR, P = 1u << LOGP, C = V << LOGG;
    static_assert(LOGR + LOGP <= LOGL, "step beyond the tile");
    const auto at = [](uint32_t point) { return vpoint<V, LOGG>(point); };
    // bound of this step's outputs (lazy 32-bit field), else canonical-ish 2
    constexpr int kBout = IsLazyBound<F>::value ? lz_plan<R>(LzIn<first>::b0, LzIn<first>::br).bout : 2;
    if constexpr (last)
        pdl_trigger();
    // ---- read R points per item: idx = u + m U + r L/R
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t idx = u + m * U + r * TS;
            T t[V];
            if constexpr (first) {
                if constexpr (COL) {
                    v16_ldg<T, V>(t, geo.src[0] + idx * geo.istride);
                } else {
#pragma unroll
                    for (int i = 0; i < V; ++i)
                        t[i] = __ldg(geo.src[i] + idx);
                }
            } else {
                v16_load<T, V>(t, sm_g + at(idx));
            }
#pragma unroll
            for (int i = 0; i < V; ++i)
                x[i][m * R + r] = t[i];
        }
    }
    // ---- twiddle w_(R p)^(r k), k = t mod p (shared by the V lines), then the DFTs
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        if constexpr (!first) {
            const uint32_t k = (u + m * U) & (P - 1);
#pragma unroll
            for (int r = 1; r < R; ++r) {
                const typename F::TW w = __ldg(&a.twL[(r * k) << (LOGL - LOGR - LOGP)]);
#pragma unroll
                for (int i = 0; i < V; ++i)
                    x[i][m * R + r] = f.mul_tw(x[i][m * R + r], w);
            }
        }
#pragma unroll
        for (int i = 0; i < V; ++i) {
            if constexpr (IsLazyBound<F>::value)
                dft_lazy<F, R, LzIn<first>::b0, LzIn<first>::br>(f, &x[i][m * R], a.wR);
            else
                dft_reg<F, R>(f, &x[i][m * R], a.wR);
        }
    }
    if constexpr (!first && !last)
        __syncthreads();  // every read of this step precedes any write
    // ---- write output r of item t to (t - k) R + k + r p
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        const uint32_t t = u + m * U;
        const uint32_t k = t & (P - 1);
        const uint32_t base = ((t - k) << LOGR) + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t pos = base + ((uint32_t)r << LOGP);
            T v[V];
#pragma unroll
            for (int i = 0; i < V; ++i)
                v[i] = x[i][m * R + bit_reverse<LOGR>(r)];
            if constexpr (last)
                vstore_last<F, V, COL, FULL4, kBout>(a, f, geo, pos, v);
            else
                v16_store<T, V>(sm_g + at(pos), v);
        }
    }
    if constexpr (!last)
        __syncthreads();
}

// Steps S.. of the tile: one leading radix-2^(LOGL mod log2 E) step when
// needed, then radix-E steps (E = 16, or 8 for half the registers, or 4 for
// twice the threads of single small transforms).
template <class F, int V, int E, int LOGL, int LOGG, int S, bool COL, int FULL4>
__device__ __forceinline__ void vsteps(const TileArgs<F> &a, const F &f, typename F::T (&x)[V][E],
                                       typename F::T *sm_g, uint32_t u, const VGeo<typename F::T, V> &geo) {
    static_assert(E == 4 || E == 8 || E == 16, "radix-4, radix-8 or radix-16 steps");
    constexpr int LE = E == 4 ? 2 : E == 8 ? 3 : 4;
    constexpr int TAIL = LOGL % LE;
    constexpr int NS = LOGL / LE + (TAIL > 0 ? 1 : 0);
    if constexpr (S < NS) {
        constexpr int LOGR = (S == 0 && TAIL > 0) ? TAIL : LE;
        constexpr int LOGP = S == 0 ? 0 : (TAIL > 0 ? TAIL + LE * (S - 1) : LE * S);
        vstep<F, V, E, LOGL, LOGG, LOGR, LOGP, S == 0, S == NS - 1, COL, FULL4>(a, f, x, sm_g, u, geo);
        vsteps<F, V, E, LOGL, LOGG, S + 1, COL, FULL4>(a, f, x, sm_g, u, geo);
    }
}

// C = V * 2^LOGG lines per CTA, 2^LOGG * L/E threads (line group fastest).
// Requirements the host checks: every pointer 16-byte aligned, C divides the
// columns of a sub-problem (COL) or the rows of a transform (ROW), a
// multi-pass plan (no n^-1 scaling in a row pass), no fused pointwise input.
// Registers are capped per thread (the compiler otherwise keeps every
// four-step twiddle of the last step live at once, up to 220 registers for
// the 32-bit column passes at E = 16, and two CTAs of 128 threads fill an
// SM). Measured on GB300 (32-bit 2^26, Goldilocks 2^24, forward + inverse):
// E = 16: 128 registers (1.09 ms against 1.30 at 160 and 1.30 at 255);
// E = 8: 64 for 4-byte values (1.03 ms against 1.20 at 80), 80 for 8-byte
// ones (0.677 ms against 0.682 at 64; with the shift-only internal twiddles
// the full-table and row passes fit 64 registers without spills, and were
// still slower there: 0.583 against 0.575 ms).
template <int E, int W>
constexpr uint32_t vregs() {
    return E == 16 ? 128 : (W == 8 ? 80 : 64);
}
template <int E, int W, uint32_t THREADS>
constexpr uint32_t vminb() {
    return (65536 / vregs<E, W>()) / THREADS > 0 ? (65536 / vregs<E, W>()) / THREADS : 1;
}

template <class F, int V, int E, int LOGL, int LOGG, bool COL, int FULL4>
__global__ void __launch_bounds__((1u << LOGG) * ((1u << LOGL) / E),
                                  vminb<E, (int)sizeof(typename F::T), (1u << LOGG) * ((1u << LOGL) / E)>())
    tile_kernel_v(const TileArgs<F> a) {
    using T = typename F::T;
    static_assert(LOGL >= 5, "at least two steps");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr uint32_t G = 1u << LOGG, C = V * G;
    const uint32_t g = threadIdx.x & (G - 1), u = threadIdx.x >> LOGG;
    F f;
    f.p = a.p;
    const uint64_t line0 = (uint64_t)blockIdx.x * C + g * V;  // the thread's first line over the batch
    const uint32_t logPer = a.logN - LOGL;                     // lines per transform
    const uint64_t b = line0 >> logPer;
    const uint64_t rem = line0 & ((1ull << logPer) - 1);
    const T *ibase = a.in + (b << a.logN);
    T *obase = a.out + (b << a.logN);
    VGeo<T, V> geo;
    if constexpr (COL) {
        const uint64_t q = rem >> a.logS;
        geo.col0 = (uint32_t)(rem & ((1ull << a.logS) - 1));
        geo.src[0] = ibase + (q << a.logM) + geo.col0;
#pragma unroll
        for (int i = 1; i < V; ++i)
            geo.src[i] = geo.src[0];
        geo.dst = obase + (q << a.logM) + geo.col0;
        geo.istride = geo.ostride = 1u << a.logS;
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) {
            const uint64_t r = rem + i;
            const uint64_t inrow = ((r & ((1ull << a.logN1) - 1)) << a.logN2) + (r >> a.logN1);
            geo.src[i] = ibase + (inrow << LOGL);
        }
        geo.dst = obase + rem;
        geo.istride = 1;
        geo.ostride = 1u << logPer;
        geo.col0 = 0;
    }
    pdl_enter();
    T x[V][E];
    vsteps<F, V, E, LOGL, LOGG, 0, COL, FULL4>(a, f, x, reinterpret_cast<T *>(smem_raw) + g * V, u, geo);
}

}  // namespace stntt
