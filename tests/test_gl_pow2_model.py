"""The Goldilocks multiply-by-2^e sequences of FieldGL::mul_pow2
(stntt_gb300/csrc/fields.cuh), restated op for op on 32-bit limbs and checked
against exact arithmetic for every exponent the kernels use (0 < e < 96) on
limb-boundary and random 64-bit inputs (no GPU). The GPU parity tests check
the kernels themselves."""

import random

P = (1 << 64) - (1 << 32) + 1
M32 = 0xFFFFFFFF


def _sub_fix(a1, a0, b1, b0):
    # (a1:a0) - (b1:b0) mod 2^64; on borrow subtract 2^32 - 1 (adds p mod 2^64)
    v = ((a1 << 32) | a0) - ((b1 << 32) | b0)
    if v < 0:
        v += 1 << 64
        v -= M32
    return v


def mul_pow2(x, e):
    x0, x1 = x & M32, x >> 32
    s = e & 31
    z0 = (x0 << s) & M32
    z1 = (((x1 << s) | (x0 >> (32 - s))) & M32) if s else x1  # funnel shift
    z2 = (x1 >> (32 - s)) if s else 0
    if e < 32:  # (z1:z0) - (~z2 * 2^32 + z2 + 1)
        assert z2 + 1 <= M32
        return _sub_fix(z1, z0, (~z2) & M32, z2 + 1)
    if e < 64:  # ((z0 + z1 mod 2^32) + c) 2^32 - (z1 + z2 + c)
        t = z0 + z1
        c = t >> 32
        a1 = (t & M32) + c
        assert a1 <= M32
        b = z1 + z2 + c
        return _sub_fix(a1, 0, b >> 32, b & M32)
    b = z0 + z1  # z0 2^32 - (z2 2^32 + z0 + z1)
    return _sub_fix(z0, 0, (b >> 32) + z2, b & M32)


def test_sixteenth_roots_are_powers_of_two():
    w16 = pow(7, (P - 1) // 16, P)
    assert w16 == pow(2, 156, P) and pow(w16, P - 2, P) == pow(2, 36, P)
    for q in range(1, 8):  # w_16^q = (-1)^(e >= 96) 2^(e mod 96)
        for base, w in ((156, w16), (36, pow(w16, P - 2, P))):
            e = base * q % 192
            assert pow(w, q, P) == (P - pow(2, e % 96, P) if e >= 96 else pow(2, e, P))


def test_mul_pow2_model_exact():
    rnd = random.Random(7)
    xs = [0, 1, 2, P - 2, P - 1, P, P + 1, (1 << 64) - 1, 1 << 63, (1 << 32) - 1, 1 << 32, M32 << 32,
          (M32 << 32) | 1] + [rnd.getrandbits(64) for _ in range(3000)]
    for e in range(1, 96):
        w = pow(2, e, P)
        for x in xs:
            r = mul_pow2(x, e)
            assert 0 <= r < P and r == x * w % P, (e, x)
