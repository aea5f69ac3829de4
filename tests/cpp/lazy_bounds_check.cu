// Host check of the compile-time bound plans of the 32-bit vector-lines DFTs
// (lz_plan / dft_lazy in stntt_gb300/csrc/tile_v.cuh). For every radix and
// input-bound pair the steps use, it replays the planned network in 64-bit
// arithmetic with worst-case and random inputs below their bounds, products
// at the top of their [0, 2p) range, and checks that (a) every halving input
// lies below 2K p, (b) every sum and difference stays below 8p (so the
// 32-bit kernel never wraps), (c) every output lies below the plan's bout,
// and (d) the outputs are congruent to the exact DIF network mod p; and
// that the Shoup and Montgomery products keep inputs below 8p in [0, 2p).
// Prints the violations it finds and a summary line; exits non-zero on any.
#include <cstdint>
#include <cstdio>
#include <random>

#include "tile_v.cuh"

using namespace stntt;

static uint64_t powmod(uint64_t b, uint64_t e, uint64_t p) {
    uint64_t r = 1;
    b %= p;
    while (e) {
        if (e & 1)
            r = r * b % p;
        b = b * b % p;
        e >>= 1;
    }
    return r;
}

// a primitive 16th root of unity mod p (p - 1 divisible by 16), or 1 for
// small primes whose 2-adic order is lower (only congruence is checked)
static uint64_t root16(uint64_t p) {
    if ((p - 1) % 16 != 0)
        return 1;
    for (uint64_t g = 2; g < p; ++g) {
        const uint64_t w = powmod(g, (p - 1) / 16, p);
        if (powmod(w, 8, p) == p - 1)
            return w;
    }
    return 1;
}

template <int R>
static int run(uint64_t p, int b0, int br, std::mt19937_64 &rng, int trials) {
    constexpr int LV = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
    const LzPlan<R> P = lz_plan<R>(b0, br);
    int bad = 0;
    if (P.bout < 1 || P.bout > 8) {
        std::printf("R=%d b0=%d br=%d: no plan\n", R, b0, br);
        return 1;
    }
    uint64_t w16[16];
    const uint64_t w = root16(p);
    for (int i = 0; i < 16; ++i)
        w16[i] = powmod(w, i, p);
    for (int t = 0; t < trials; ++t) {
        uint64_t x[16], y[16];
        for (int i = 0; i < R; ++i) {
            const uint64_t B = i == 0 ? b0 : br;
            const uint64_t v = t % 4 == 0 ? B * p - 1 - rng() % 3 : rng() % (B * p);
            x[i] = v;
            y[i] = v % p;
        }
        for (int L = 0, h = R / 2; L < LV; ++L, h /= 2) {
            int q = 0;
            for (int base = 0; base < R; base += 2 * h) {
                for (int j = 0; j < h; ++j, ++q) {
                    const int a = base + j, b = a + h;
                    for (int side = 0; side < 2; ++side) {
                        const uint64_t k = side ? P.rb[L][q] : P.ra[L][q];
                        uint64_t &v = side ? x[b] : x[a];
                        if (k) {
                            bad += v >= 2 * k * p;
                            if (v >= k * p)
                                v -= k * p;
                        }
                    }
                    const uint64_t K = P.kd[L][q];
                    bad += x[b] > K * p;
                    const uint64_t s = x[a] + x[b], d = x[a] + K * p - x[b];
                    bad += s >= 8 * p || d >= 8 * p || s >= (1ull << 32) || d >= (1ull << 32);
                    x[a] = s;
                    if (j == 0) {
                        x[b] = d;
                    } else {
                        const uint64_t c = d % p * w16[j * (16 / (2 * h))] % p;
                        x[b] = c + (t % 2 ? p : 0);  // a Shoup product lies in [0, 2p): also its top
                    }
                    const uint64_t ya = y[a], yb = y[b];
                    y[a] = (ya + yb) % p;
                    y[b] = (ya + p - yb) % p;
                    if (j != 0)
                        y[b] = y[b] * w16[j * (16 / (2 * h))] % p;
                }
            }
        }
        for (int i = 0; i < R; ++i)
            bad += x[i] >= (uint64_t)P.bout * p || x[i] % p != y[i];
    }
    if (bad)
        std::printf("p=%llu R=%d b0=%d br=%d bout=%d: %d violations\n", (unsigned long long)p, R, b0, br, P.bout,
                    bad);
    return bad;
}

// canonicalisation of a value below B p by the halving sequence of
// FieldU32L::canon_b (K = 4, 2, 1 where B > 2K ... B > K)
static int canon_check(uint64_t p) {
    int bad = 0;
    for (int B = 1; B <= 8; ++B) {
        for (uint64_t v : {uint64_t(0), p - 1, p, 2 * p - 1, 3 * p + 5, B * p - 1}) {
            if (v >= B * p)
                continue;
            uint64_t a = v;
            if (B > 4 && a >= 4 * p)
                a -= 4 * p;
            if (B > 2 && a >= 2 * p)
                a -= 2 * p;
            if (B > 1 && a >= p)
                a -= p;
            bad += a >= p || a != v % p;
        }
    }
    return bad;
}

// The two products the steps apply to values below 8p, restated from
// FieldU32L (fields.cuh): Shoup's a*w - floor(a*w'/2^32)*p for any 32-bit a,
// and Montgomery's REDC(a * (w 2^32 mod p)) for a < 8p. Both must land in
// [0, 2p) and be congruent to a*w.
static int product_check(uint64_t p, std::mt19937_64 &rng) {
    int bad = 0;
    uint32_t pinv = (uint32_t)p;  // -p^-1 mod 2^32 by Newton's iteration
    for (int i = 0; i < 4; ++i)
        pinv *= 2u - (uint32_t)p * pinv;
    pinv = 0u - pinv;
    for (int t = 0; t < 20000; ++t) {
        const uint64_t w = rng() % p;
        const uint32_t wsh = (uint32_t)((w << 32) / p);
        const uint32_t a32 = t % 3 == 0 ? 0xffffffffu - (uint32_t)(rng() % 4) : (uint32_t)rng();
        const uint32_t q = (uint32_t)(((uint64_t)a32 * wsh) >> 32);
        const uint32_t r = a32 * (uint32_t)w - q * (uint32_t)p;
        bad += r >= 2 * p || r % p != (uint64_t)a32 * w % p;
        const uint64_t a = t % 3 == 0 ? 8 * p - 1 - rng() % 4 : rng() % (8 * p);
        const uint32_t wr = (uint32_t)((w << 32) % p);
        const uint32_t lo = (uint32_t)a * wr, hi = (uint32_t)((a * wr) >> 32);
        const uint32_t m = lo * pinv;
        const uint64_t red = (uint64_t)hi + (((uint64_t)m * p) >> 32) + (lo != 0u);
        bad += red >= 2 * p || red % p != a * w % p;
    }
    return bad;
}

int main() {
    std::mt19937_64 rng(12345);
    // every findParams prime up to n = 2^26 and the largest prime below 2^29
    const uint64_t primes[] = {17, 257, 7681, 12289, 40961, 65537, 786433, 5767169, 7340033, 23068673,
                               104857601, 167772161, 469762049, 536870909};
    int bad = 0;
    for (uint64_t p : primes) {
        bad += canon_check(p);
        bad += product_check(p, rng);
        for (int first = 0; first < 2; ++first) {
            const int b0 = first ? LzIn<true>::b0 : LzIn<false>::b0, br = first ? LzIn<true>::br : LzIn<false>::br;
            bad += run<2>(p, b0, br, rng, 2000);
            bad += run<4>(p, b0, br, rng, 2000);
            bad += run<8>(p, b0, br, rng, 2000);
            bad += run<16>(p, b0, br, rng, 2000);
        }
    }
    std::printf("plans R=2/4/8/16: bout %d/%d/%d/%d (later steps), %d/%d/%d/%d (first); violations %d\n",
                lz_plan<2>(8, 2).bout, lz_plan<4>(8, 2).bout, lz_plan<8>(8, 2).bout, lz_plan<16>(8, 2).bout,
                lz_plan<2>(1, 1).bout, lz_plan<4>(1, 1).bout, lz_plan<8>(1, 1).bout, lz_plan<16>(1, 1).bout, bad);
    return bad != 0;
}
