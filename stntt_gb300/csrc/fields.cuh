// fields.cuh -- modular arithmetic for the two NTT fields (device side).
//
// FieldU32: a runtime prime p < 2^31 (the reference's per-size prime from
//   findParams, src/ntt/ntt_util.cpp:10-49). Replaces the reference's
//   butterfly with three runtime '%' (src/cuda/ntt/arithmetic.cuh:17-24,
//   src/cuda/math.cuh:10-16). Twiddles are Shoup pairs (w, floor(w*2^32/p)),
//   so a twiddle product costs one mul.hi and two mul.lo.
// FieldGL: Goldilocks p = 2^64 - 2^32 + 1. The reference has add/sub only
//   (src/cuda/ntt/implementations/goldilocks/arithmetic.cuh:19-30; mul and
//   butterfly are empty at :32-35). Products are 64x64->128 mad.lo/mad.hi
//   chains reduced with 2^64 = 2^32 - 1 and 2^96 = -1 (mod p).
// All values are kept canonical (< p).
#pragma once
#include <cstdint>
#include <type_traits>

namespace stntt {

struct FieldU32 {
    using T = uint32_t;
    using TW = uint2;  // {w, floor(w * 2^32 / p)}
    uint32_t p;

    __device__ __forceinline__ T add(T a, T b) const {
        uint32_t s = a + b;
        return min(s, s - p);
    }
    __device__ __forceinline__ T sub(T a, T b) const {
        uint32_t d = a - b + p;
        return min(d, d - p);
    }
    // Shoup: q = floor(a * w' / 2^32); a*w - q*p lies in [0, 2p).
    __device__ __forceinline__ T mul_tw(T a, TW w) const {
        uint32_t q = __umulhi(a, w.y);
        uint32_t r = a * w.x - q * p;
        return min(r, r - p);
    }
    // General product of two residues (pointwise products).
    __device__ __forceinline__ T mul(T a, T b) const { return (uint32_t)(((uint64_t)a * b) % p); }
    __device__ __forceinline__ static T tw_value(TW w) { return w.x; }
    // difference that only feeds a twiddle product; canonical form for storing
    __device__ __forceinline__ T sub_lazy(T a, T b) const { return sub(a, b); }
    __device__ __forceinline__ T canon(T a) const { return a; }
};

// The same field for p < 2^30 with lazy reduction (Harvey's butterflies):
// values rest in [0, 2p); a difference that feeds a product is a - b + 2p in
// [0, 4p) (one add); Shoup products of any input below 2^32 land in [0, 2p)
// without a correction; canon() maps [0, 2p) to [0, p) before HBM stores.
struct FieldU32L {
    using T = uint32_t;
    using TW = uint2;
    uint32_t p;

    __device__ __forceinline__ T add(T a, T b) const {
        const uint32_t s = a + b;
        return min(s, s - 2 * p);
    }
    __device__ __forceinline__ T sub(T a, T b) const {
        const uint32_t d = a - b + 2 * p;
        return min(d, d - 2 * p);
    }
    __device__ __forceinline__ T sub_lazy(T a, T b) const { return a - b + 2 * p; }
    __device__ __forceinline__ T mul_tw(T a, TW w) const {
        const uint32_t q = __umulhi(a, w.y);
        return a * w.x - q * p;
    }
    __device__ __forceinline__ T mul(T a, T b) const { return (uint32_t)(((uint64_t)a * b) % p); }
    __device__ __forceinline__ static T tw_value(TW w) { return w.x; }
    __device__ __forceinline__ T canon(T a) const { return min(a, a - p); }
    // a * w for a table entry wr = w * 2^32 mod p (Montgomery form, 4 bytes
    // instead of a Shoup pair's 8): REDC(a * wr) with pinv = -p^-1 mod 2^32.
    // For a < 2p, wr < p: (a wr + m p) / 2^32 < 2p, so the result rests in
    // [0, 2p) like every lazy value; lo + (m p mod 2^32) is 0 or 2^32.
    __device__ __forceinline__ T mul_mont(T a, uint32_t wr, uint32_t pinv) const {
        const uint32_t lo = a * wr, hi = __umulhi(a, wr);
        const uint32_t m = lo * pinv;
        return hi + __umulhi(m, p) + (lo != 0u);
    }
    // Wider headroom for p < 2^29 (8p < 2^32), used by the vector-lines DFT
    // (dft_lazy): a value below B p with B <= 8 stays a 32-bit number, a
    // Shoup product of it still lands in [0, 2p), and so does a Montgomery
    // product (a wr + m p) / 2^32 < (8p^2 + 2^32 p) / 2^32 < 2p.
    // red(a, K): a in [0, 2K p) -> [0, K p) (one conditional subtraction).
    __device__ __forceinline__ T red(T a, uint32_t k) const { return min(a, a - k * p); }
    // a in [0, B p) -> [0, p) by halving steps.
    template <int B>
    __device__ __forceinline__ T canon_b(T a) const {
        if constexpr (B > 4)
            a = red(a, 4);
        if constexpr (B > 2)
            a = red(a, 2);
        if constexpr (B > 1)
            a = red(a, 1);
        return a;
    }
};

// Fields whose vector-lines steps track value bounds (FieldU32L with p < 2^29).
template <class F>
struct IsLazyBound : std::false_type {};
template <>
struct IsLazyBound<FieldU32L> : std::true_type {};

struct FieldGL {
    using T = uint64_t;
    using TW = uint64_t;
    static constexpr uint64_t P = 0xFFFFFFFF00000001ull;
    uint32_t p;  // unused; keeps the two field types interchangeable

    __device__ __forceinline__ T add(T a, T b) const {
        // a + b = a - (p - b): p - b lies in [1, p], so the subtraction below
        // (one conditional + p on borrow) returns a canonical value. Seven
        // integer ops against nine for an add with a carry fix and a compare.
        uint32_t s0, s1;
        asm("{\n\t"
            ".reg .u32 n0, n1, m;\n\t"
            "sub.cc.u32 n0, 1, %4;\n\t"
            "subc.u32 n1, 0xffffffff, %5;\n\t"
            "sub.cc.u32 %0, %2, n0;\n\t"
            "subc.cc.u32 %1, %3, n1;\n\t"
            "subc.u32 m, 0, 0;\n\t"
            "sub.cc.u32 %0, %0, m;\n\t"
            "subc.u32 %1, %1, 0;\n\t"
            "}"
            : "=&r"(s0), "=&r"(s1)
            : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
        return ((uint64_t)s1 << 32) | s0;
    }

    __device__ __forceinline__ T sub(T a, T b) const {
        // d = a - b; on borrow d += p, i.e. d -= 2^32 - 1 (mod 2^64).
        uint32_t d0, d1;
        asm("{\n\t"
            ".reg .u32 m;\n\t"
            "sub.cc.u32 %0, %2, %4;\n\t"
            "subc.cc.u32 %1, %3, %5;\n\t"
            "subc.u32 m, 0, 0;\n\t"
            "sub.cc.u32 %0, %0, m;\n\t"
            "subc.u32 %1, %1, 0;\n\t"
            "}"
            : "=&r"(d0), "=&r"(d1)
            : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
        return ((uint64_t)d1 << 32) | d0;
    }

    __device__ __forceinline__ T mul(T a, T b) const {
        uint32_t r0, r1;
        asm("{\n\t"
            ".reg .u32 r2, r3, t0, t1, m, u0, u1;\n\t"
            // 128-bit product (r3:r2:r1:r0) = a * b
            "mul.lo.u32 %0, %2, %4;\n\t"
            "mul.hi.u32 %1, %2, %4;\n\t"
            "mad.lo.cc.u32 %1, %2, %5, %1;\n\t"
            "madc.hi.u32 r2, %2, %5, 0;\n\t"
            "mad.lo.cc.u32 %1, %3, %4, %1;\n\t"
            "madc.hi.cc.u32 r2, %3, %4, r2;\n\t"
            "madc.hi.u32 r3, %3, %5, 0;\n\t"
            "mad.lo.cc.u32 r2, %3, %5, r2;\n\t"
            "addc.u32 r3, r3, 0;\n\t"
            // t = (r1:r0) - r3; on borrow add p (i.e. subtract 2^32 - 1)
            "sub.cc.u32 t0, %0, r3;\n\t"
            "subc.cc.u32 t1, %1, 0;\n\t"
            "subc.u32 m, 0, 0;\n\t"
            "sub.cc.u32 t0, t0, m;\n\t"
            "subc.u32 t1, t1, 0;\n\t"
            // u = r2 * (2^32 - 1) <= (2^32 - 1)^2; result = t + u = t - (p - u).
            // p - u = (~r2 + k) * 2^32 + (r2 + 1), k the carry of r2 + 1; both
            // limbs as multiply-adds (r2 * 1 + 1, r2 * (2^32 - 1) + 2^32 - 1 = ~r2),
            // which run on the FMA pipe beside the ALU-bound carry chains.
            "mad.lo.cc.u32 u0, r2, 1, 1;\n\t"
            "madc.lo.u32 u1, r2, 0xffffffff, 0xffffffff;\n\t"
            // t + u < 2p, so one conditional + p on borrow leaves it canonical
            "sub.cc.u32 %0, t0, u0;\n\t"
            "subc.cc.u32 %1, t1, u1;\n\t"
            "subc.u32 m, 0, 0;\n\t"
            "sub.cc.u32 %0, %0, m;\n\t"
            "subc.u32 %1, %1, 0;\n\t"
            "}"
            : "=&r"(r0), "=&r"(r1)
            : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
        return ((uint64_t)r1 << 32) | r0;
    }
    __device__ __forceinline__ T mul_tw(T a, TW w) const { return mul(a, w); }
    __device__ __forceinline__ static T tw_value(TW w) { return w; }
    __device__ __forceinline__ T sub_lazy(T a, T b) const { return sub(a, b); }
    __device__ __forceinline__ T canon(T a) const { return a; }

    // x * 2^e mod p for 0 < e < 96 (any 64-bit x; canonical result), with e
    // a constant once the caller's loops are unrolled. The 16th roots of
    // unity mod p are powers of two (2 has order 192: w_16 = 2^(12 k), k
    // odd), so the radix-16/8/4 internal twiddles need no product: shift x
    // into limbs (z2:z1:z0 = x * 2^s, s = e mod 32) and fold the limbs above
    // 2^64 back with 2^64 = 2^32 - 1 and 2^96 = -1. 10 integer ops for e < 32
    // or e >= 64, 15 for 32 <= e < 64, against 21 for a product.
    __device__ __forceinline__ T mul_pow2(T x, int e) const {
        const uint32_t x0 = (uint32_t)x, x1 = (uint32_t)(x >> 32);
        const int s = e & 31;
        const uint32_t z0 = x0 << s;
        const uint32_t z1 = s ? __funnelshift_l(x0, x1, s) : x1;
        const uint32_t z2 = s ? x1 >> (32 - s) : 0u;
        uint32_t r0, r1;
        if (e < 32) {
            // (z1:z0) + z2 (2^32 - 1) = (z1:z0) - (p - z2 (2^32 - 1)), and
            // p - z2 (2^32 - 1) = ~z2 * 2^32 + (z2 + 1) for z2 < 2^31
            asm("{\n\t"
                ".reg .u32 m;\n\t"
                "sub.cc.u32 %0, %2, %4;\n\t"
                "subc.cc.u32 %1, %3, %5;\n\t"
                "subc.u32 m, 0, 0;\n\t"
                "sub.cc.u32 %0, %0, m;\n\t"
                "subc.u32 %1, %1, 0;\n\t"
                "}"
                : "=&r"(r0), "=&r"(r1)
                : "r"(z0), "r"(z1), "r"(z2 + 1u), "r"(~z2));
        } else if (e < 64) {
            // z 2^32 = z0 2^32 + z1 2^64 + z2 2^96 = (z0 + z1) 2^32 - z1 - z2;
            // with c the carry of z0 + z1 (worth 2^64 = 2^32 - 1):
            // ((z0 + z1 mod 2^32) + c) 2^32 - (z1 + z2 + c), no limb overflows
            asm("{\n\t"
                ".reg .u32 sl, c, a1, b0, b1, m;\n\t"
                "add.cc.u32 sl, %2, %3;\n\t"
                "addc.u32 c, 0, 0;\n\t"
                "add.u32 a1, sl, c;\n\t"
                "add.cc.u32 b0, %3, %4;\n\t"
                "addc.u32 b1, 0, 0;\n\t"
                "add.cc.u32 b0, b0, c;\n\t"
                "addc.u32 b1, b1, 0;\n\t"
                "sub.cc.u32 %0, 0, b0;\n\t"
                "subc.cc.u32 %1, a1, b1;\n\t"
                "subc.u32 m, 0, 0;\n\t"
                "sub.cc.u32 %0, %0, m;\n\t"
                "subc.u32 %1, %1, 0;\n\t"
                "}"
                : "=&r"(r0), "=&r"(r1)
                : "r"(z0), "r"(z1), "r"(z2));
        } else {
            // z 2^64 = z0 2^64 + z1 2^96 + z2 2^128 = z0 2^32 - (z2 2^32 + z0 + z1)
            asm("{\n\t"
                ".reg .u32 b0, b1, m;\n\t"
                "add.cc.u32 b0, %2, %3;\n\t"
                "addc.u32 b1, %4, 0;\n\t"
                "sub.cc.u32 %0, 0, b0;\n\t"
                "subc.cc.u32 %1, %2, b1;\n\t"
                "subc.u32 m, 0, 0;\n\t"
                "sub.cc.u32 %0, %0, m;\n\t"
                "subc.u32 %1, %1, 0;\n\t"
                "}"
                : "=&r"(r0), "=&r"(r1)
                : "r"(z0), "r"(z1), "r"(z2));
        }
        return ((uint64_t)r1 << 32) | r0;
    }
};

// Goldilocks with the transform's radix-16 root fixed at compile time, so
// that the internal twiddles of the register DFTs are shifts (mul_pow2):
// DIR = +1 for w_16 = 7^((p-1)/16) = 2^156 (every forward transform: the root
// of 2^k points is 7^((p-1)/2^k)), -1 for its inverse 2^36. The host picks
// these types only when a pass's w_16 is that value.
template <int DIR>
struct FieldGLPow2 : FieldGL {
    static constexpr int kDir = DIR;
    // w_16^q = (-1)^neg 2^e, e < 96, for q = 1..7
    __device__ __forceinline__ static constexpr int w16_exp(int q) {
        return ((DIR > 0 ? 156 : 36) * q) % 192;
    }
};
using FieldGLF = FieldGLPow2<1>;
using FieldGLI = FieldGLPow2<-1>;

template <class F>
struct IsPow2Field : std::false_type {};
template <int DIR>
struct IsPow2Field<FieldGLPow2<DIR>> : std::true_type {};

}  // namespace stntt
