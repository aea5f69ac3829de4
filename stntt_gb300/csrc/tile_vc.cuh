// tile_vc.cuh -- the vector-lines pass with each line's DFT spread over the
// K CTAs of a thread-block cluster, for 2^12- and 2^13-point passes: the
// two-HBM-pass plans of 2^24 (Goldilocks) and 2^26 (32-bit) points.
//
// A tile is C adjacent lines (columns of a column pass, rows of a row pass)
// of L = L1 * L2 points. Point j = j1 * L2 + j2 of a line; output k = k1 +
// L1 * k2. The line's DFT is done in two phases inside the cluster (the
// four-step split of tile.cuh once more, in shared memory):
//   phase 1: CTA r takes j2 in [r Q, (r+1) Q), Q = L2 / K: the L1-point DFTs
//     over j1 of its Q * C sub-lines, loaded from HBM (16 bytes = V lines per
//     access, as in tile_v.cuh), each output k1 multiplied by w_L^(j2 k1) and
//     left in its own shared memory, point-major [k1][q][C];
//   cluster barrier (every CTA's phase-1 results complete and visible;
//     arrive and wait split around the phase-2 set-up);
//   phase 2: CTA r takes k1 in [r P, (r+1) P), P = L1 / K: the L2-point DFTs
//     over j2, whose inputs (k1, j2) sit in CTA j2 / Q's shared memory and are
//     read through distributed shared memory, 16 bytes per access; after
//     those reads a second cluster barrier (arrive after the reads, wait
//     after the first DFTs) lets every CTA reuse its buffer for the rest of
//     phase 2; outputs k = k1 + L1 k2 go to HBM as the
//     vector-lines pass writes them (four-step twiddle of a column pass,
//     digit-reversed positions of a row pass).
// Shared memory per CTA: L * C * w / K bytes; both phases' tiles share it.
// Every CTA of a cluster runs the same steps and reaches both barriers (no
// early exit; the host launches whole clusters over whole tiles).
#pragma once
#include <cstdint>

#include "tile_v.cuh"

namespace stntt {

__device__ __forceinline__ uint32_t vc_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// The cluster barrier, for every thread of every CTA of the cluster; it
// orders shared-memory accesses across the cluster (release on arrive,
// acquire on wait). Work between the arrive and the wait overlaps the other
// CTAs' arrival.
__device__ __forceinline__ void vc_cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void vc_cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// 16 bytes (V elements) from CTA `rank`'s shared memory at the offset of the
// local address p.
template <class T, int V>
__device__ __forceinline__ void v16_load_cluster(T (&x)[V], const T *p, uint32_t rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t ra, w0, w1, w2, w3;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    asm volatile("ld.shared::cluster.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(w0), "=r"(w1), "=r"(w2), "=r"(w3)
                 : "r"(ra)
                 : "memory");
    if constexpr (sizeof(T) == 4) {
        static_assert(V == 4, "16 bytes of 4-byte values");
        x[0] = w0, x[1] = w1, x[2] = w2, x[3] = w3;
    } else {
        static_assert(V == 2, "16 bytes of 8-byte values");
        x[0] = ((uint64_t)w1 << 32) | w0;
        x[1] = ((uint64_t)w3 << 32) | w2;
    }
}

// One radix-2^LOGR Stockham step of an L_S = 2^LOGS-point sub-DFT over the
// tile (see vstep in tile_v.cuh). The step twiddles w_(L_S)^e come from the
// pass's w_L table at e << TWS. FIRST reads through load(idx, t), LAST writes
// through store(pos, v), the others use the shared-memory tile. SYNC between
// this step's reads and its writes: 0 none, 1 the CTA, 2 the cluster (its
// arrive right after the reads, its wait before the writes).
template <class F, int V, int E, int LOGS, int LOGGT, int LOGR, int LOGP, int TWS, bool FIRST, bool LAST, int SYNC,
          class LOAD, class STORE>
__device__ __forceinline__ void vcstep(const TileArgs<F> &a, const F &f, typename F::T (&x)[V][E],
                                       typename F::T *sm_g, uint32_t u, const LOAD &load, const STORE &store) {
    using T = typename F::T;
    constexpr int R = 1 << LOGR, ITEMS = E / R;
    constexpr uint32_t U = (1u << LOGS) / E, TS = (1u << LOGS) >> LOGR, P = 1u << LOGP;
    static_assert(LOGR + LOGP <= LOGS, "step beyond the sub-DFT");
    const auto at = [](uint32_t point) { return vpoint<V, LOGGT>(point); };
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t idx = u + m * U + r * TS;
            T t[V];
            if constexpr (FIRST)
                load(idx, t);
            else
                v16_load<T, V>(t, sm_g + at(idx));
#pragma unroll
            for (int i = 0; i < V; ++i)
                x[i][m * R + r] = t[i];
        }
    }
    if constexpr (SYNC == 2)
        vc_cluster_arrive();  // this thread's reads are done (release); the DFTs below overlap the others
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        if constexpr (!FIRST) {
            const uint32_t k = (u + m * U) & (P - 1);
#pragma unroll
            for (int r = 1; r < R; ++r) {
                const typename F::TW w = __ldg(&a.twL[((r * k) << (LOGS - LOGR - LOGP)) << TWS]);
#pragma unroll
                for (int i = 0; i < V; ++i)
                    x[i][m * R + r] = f.mul_tw(x[i][m * R + r], w);
            }
        }
#pragma unroll
        for (int i = 0; i < V; ++i)
            dft_reg<F, R>(f, &x[i][m * R], a.wR);
    }
    if constexpr (SYNC == 1)
        __syncthreads();
    else if constexpr (SYNC == 2)
        vc_cluster_wait();
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
            if constexpr (LAST)
                store(pos, v);
            else
                v16_store<T, V>(sm_g + at(pos), v);
        }
    }
    if constexpr (!LAST)
        __syncthreads();
}

// Steps S.. of an L_S-point sub-DFT (radix 2^(LOGS mod 3) first when needed,
// then radix 8): SYNC0 after the first step's reads (0 or 2), SYNCL after the
// last step's reads (1 when it writes shared memory, else 0); TRIG: the last
// step lets the next launch start (programmatic dependent launch).
template <class F, int V, int E, int LOGS, int LOGGT, int TWS, int SYNC0, int SYNCL, bool TRIG, int S, class LOAD,
          class STORE>
__device__ __forceinline__ void vcsteps(const TileArgs<F> &a, const F &f, typename F::T (&x)[V][E],
                                        typename F::T *sm_g, uint32_t u, const LOAD &load, const STORE &store) {
    static_assert(E == 8, "8 points per line");
    constexpr int LE = 3, TAIL = LOGS % LE, NS = LOGS / LE + (TAIL > 0 ? 1 : 0);
    static_assert(NS >= 2, "at least two steps per phase");
    if constexpr (S < NS) {
        constexpr int LOGR = (S == 0 && TAIL > 0) ? TAIL : LE;
        constexpr int LOGP = S == 0 ? 0 : (TAIL > 0 ? TAIL + LE * (S - 1) : LE * S);
        constexpr int SYNC = S == 0 ? SYNC0 : (S == NS - 1 ? SYNCL : 1);
        if constexpr (TRIG && S == NS - 1)
            pdl_trigger();
        vcstep<F, V, E, LOGS, LOGGT, LOGR, LOGP, TWS, S == 0, S == NS - 1, SYNC>(a, f, x, sm_g, u, load, store);
        vcsteps<F, V, E, LOGS, LOGGT, TWS, SYNC0, SYNCL, TRIG, S + 1>(a, f, x, sm_g, u, load, store);
    }
}

// L = 2^LOGL points per line, L1 = 2^LOG1, C = V * 2^LOGG lines per
// cluster, K = 2^LOGK CTAs per cluster, 8 points per line per thread.
template <int LOGL, int LOG1, int LOGG, int LOGK, int V>
__host__ __device__ constexpr uint32_t vc_threads() {
    return (1u << (LOGL - LOG1 - LOGK + LOGG)) * ((1u << LOG1) / 8);
}

template <class F, int V, int LOGL, int LOG1, int LOGG, int LOGK, bool COL, int FULL4>
__global__ void __launch_bounds__(vc_threads<LOGL, LOG1, LOGG, LOGK, V>(),
                                  vminb<8, (int)sizeof(typename F::T), vc_threads<LOGL, LOG1, LOGG, LOGK, V>()>())
    tile_kernel_vc(const TileArgs<F> a) {
    using T = typename F::T;
    constexpr int E = 8, LOG2 = LOGL - LOG1;
    constexpr int LOGQ = LOG2 - LOGK, LOGP = LOG1 - LOGK;  // sub-DFTs per CTA: phase 1 (j2), phase 2 (k1)
    static_assert(LOGQ >= 0 && LOGP >= 0, "K divides both factors");
    constexpr int LOGG1 = LOGQ + LOGG, LOGG2 = LOGP + LOGG;  // line groups of the two phase tiles
    static_assert(LOGG1 >= 2 && LOGG2 >= 2, "unpadded phase tiles");
    constexpr uint32_t G = 1u << LOGG, C = V * G, Q = 1u << LOGQ;
    constexpr uint32_t THREADS = vc_threads<LOGL, LOG1, LOGG, LOGK, V>();
    static_assert(THREADS == (1u << LOGG2) * ((1u << LOG2) / E), "both phases use every thread");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    F f;
    f.p = a.p;
    const uint32_t rank = vc_rank();
    const uint64_t line0 = (uint64_t)(blockIdx.x >> LOGK) * C;  // the tile's first line over the batch
    const uint32_t logPer = a.logN - LOGL;                       // lines per transform
    const uint64_t b = line0 >> logPer;
    const uint64_t rem = line0 & ((1ull << logPer) - 1);
    const T *ibase = a.in + (b << a.logN);
    T *obase = a.out + (b << a.logN);

    // ---- phase 1: thread = (u1, q, g); sub-line (j2 = rank Q + q, lines g V ..)
    const uint32_t g1 = threadIdx.x & ((1u << LOGG1) - 1), u1 = threadIdx.x >> LOGG1;
    const uint32_t q = g1 >> LOGG, gq = g1 & (G - 1);
    const uint32_t j2 = (rank << LOGQ) + q;
    const T *src[V];
    if constexpr (COL) {
        const uint64_t sub = rem >> a.logS;
        const uint32_t col0 = (uint32_t)(rem & ((1ull << a.logS) - 1));
        src[0] = ibase + (sub << a.logM) + col0 + gq * V;
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) {
            const uint64_t r = rem + gq * V + i;
            const uint64_t inrow = ((r & ((1ull << a.logN1) - 1)) << a.logN2) + (r >> a.logN1);
            src[i] = ibase + (inrow << LOGL);
        }
    }
    const uint32_t istride = COL ? (1u << a.logS) : 1u;
    const auto load1 = [&](uint32_t j1, T(&t)[V]) {
        const uint32_t j = (j1 << LOG2) + j2;  // point of the line, < L
        if constexpr (COL) {
            v16_ldg<T, V>(t, src[0] + j * istride);  // j * S < M <= 2^32
        } else {
#pragma unroll
            for (int i = 0; i < V; ++i)
                t[i] = __ldg(src[i] + j);
        }
    };
    T *sm_g1 = sm + g1 * V;
    const auto store1 = [&](uint32_t k1, T(&v)[V]) {  // w_L^(j2 k1), left in this CTA's tile
        const typename F::TW w = __ldg(&a.twL[j2 * k1]);
#pragma unroll
        for (int i = 0; i < V; ++i)
            v[i] = f.mul_tw(v[i], w);
        v16_store<T, V>(sm_g1 + vpoint<V, LOGG1>(k1), v);
    };
    pdl_enter();
    T x[V][E];
    vcsteps<F, V, E, LOG1, LOGG1, LOG2, 0, 1, false, 0>(a, f, x, sm_g1, u1, load1, store1);
    vc_cluster_arrive();  // this CTA's phase-1 results are written (release)

    // ---- phase 2: thread = (u2, p, g); line (k1 = rank P + p, lines g V ..)
    const uint32_t g2 = threadIdx.x & ((1u << LOGG2) - 1), u2 = threadIdx.x >> LOGG2;
    const uint32_t p = g2 >> LOGG, gp = g2 & (G - 1);
    const uint32_t k1 = (rank << LOGP) + p;
    // (k1, j2) of lines gp V .. in CTA j2 / Q: point k1, sub-line (j2 mod Q, gp) of its phase-1 tile
    const T *xsrc = sm + vpoint<V, LOGG1>(k1) + gp * V;
    const auto load2 = [&](uint32_t jj, T(&t)[V]) {
        v16_load_cluster<T, V>(t, xsrc + (jj & (Q - 1)) * C, jj >> LOGQ);
    };
    VGeo<T, V> geo;
    if constexpr (COL) {
        geo.col0 = (uint32_t)(rem & ((1ull << a.logS) - 1)) + gp * V;
        geo.dst = obase + ((rem >> a.logS) << a.logM) + geo.col0;
        geo.ostride = 1u << a.logS;
    } else {
        geo.col0 = 0;
        geo.dst = obase + rem + gp * V;
        geo.ostride = 1u << logPer;
    }
    const auto store2 = [&](uint32_t k2, T(&v)[V]) { vstore_last<F, V, COL, FULL4>(a, f, geo, k1 + (k2 << LOG1), v); };
    vc_cluster_wait();  // every CTA's phase-1 results are visible (acquire)
    vcsteps<F, V, E, LOG2, LOGG2, LOG1, 2, 0, true, 0>(a, f, x, sm + g2 * V, u2, load2, store2);
}

}  // namespace stntt
