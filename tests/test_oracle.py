"""The CPU oracle, pinned against vectors produced by the unmodified reference."""

import hashlib

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).astype("<i4").tobytes()).hexdigest()


def test_rng_matches_reference(golden):
    g = golden["rng"]
    s = O.ref_rng_vector(1 << 26, g["seed"])
    assert s[:64].tolist() == g["first64"]
    assert sha(s) == g["sha256_2^26"]


def test_find_params_matches_reference(golden):
    for lg, (root, mod) in golden["params"].items():
        assert O.find_params(1 << int(lg), 11) == (root, mod), lg


@pytest.mark.parametrize("maxlog", [20])
def test_ref_wrap_restatement_matches_reference(golden, maxlog):
    stream = O.ref_rng_vector(10 << 20)
    for case in golden["stockham"]:
        n, b = 1 << case["log_n"], case["batch"]
        if case["log_n"] > maxlog:
            continue
        out = O.ntt_ref_wrap(stream[: n * b], case["root"], case["mod"], batch=b)
        assert sha(out) == case["sha256"], (case["log_n"], b)
        if "out" in case:
            assert out.tolist() == case["out"]


def test_ref_wrap_restatement_large(golden):
    """The reference suite's skipped range (st_ntt_test.cu:87-97), batch 1."""
    stream = O.ref_rng_vector(1 << 24)
    for case in golden["stockham"]:
        if 20 < case["log_n"] <= 24:
            n = 1 << case["log_n"]
            out = O.ntt_ref_wrap(stream[:n], case["root"], case["mod"])
            assert sha(out) == case["sha256"], case["log_n"]


def test_exact_equals_reference_where_no_overflow(golden):
    """For n <= 2^13 (p < 46341) the reference's int32 arithmetic is exact."""
    stream = O.ref_rng_vector(10 << 13)
    checked = 0
    for case in golden["stockham"]:
        if case["log_n"] <= 13:
            n, b = 1 << case["log_n"], case["batch"]
            out = O.ntt_u32(stream[: n * b].astype(np.uint32), case["root"], case["mod"], batch=b)
            assert sha(out.view(np.int32)) == case["sha256"], (case["log_n"], b)
            checked += 1
    assert checked == 12 * 4


def test_exact_differs_from_reference_after_overflow(golden):
    """n = 2^14 onward, the reference's products overflow int32."""
    stream = O.ref_rng_vector(1 << 16)
    case = next(c for c in golden["stockham"] if c["log_n"] == 16 and c["batch"] == 1)
    out = O.ntt_u32(stream[: 1 << 16].astype(np.uint32), case["root"], case["mod"])
    assert sha(out.view(np.int32)) != case["sha256"]


@pytest.mark.parametrize("lg", list(range(0, 11)))
def test_stockham_equals_schoolbook_u32(lg):
    n = 1 << lg
    root, mod = O.find_params(n, 11)
    x = O.uniform_u32(1000 + lg, mod, n)
    assert np.array_equal(O.ntt_u32(x, root, mod), O.dft_u32(x, root, mod))


@pytest.mark.parametrize("lg", list(range(0, 11)))
def test_stockham_equals_schoolbook_gl64(lg):
    n = 1 << lg
    x = O.uniform_u64(2000 + lg, n)
    assert np.array_equal(O.ntt_gl64(x), O.dft_gl64(x, O.gl_root(lg)))


@pytest.mark.parametrize("lg", [1, 5, 12, 16, 20])
def test_round_trip(lg):
    n = 1 << lg
    root, mod = O.find_params(n, 11)
    x = O.uniform_u32(7, mod, n)
    assert np.array_equal(O.ntt_u32(O.ntt_u32(x, root, mod), root, mod, inverse=True), x)
    y = O.uniform_u64(8, n)
    assert np.array_equal(O.ntt_gl64(O.ntt_gl64(y), inverse=True), y)


def test_goldilocks_root_structure():
    P = O.GL_P
    # 7 generates the multiplicative group: 7^((P-1)/q) != 1 for every prime q | P-1
    for q in (2, 3, 5, 17, 257, 65537):
        assert (P - 1) % q == 0
        assert O.lib().orc_gl_pow(7, (P - 1) // q) != 1
    w = O.gl_root(32)
    assert O.lib().orc_gl_pow(w, 1 << 32) == 1 and O.lib().orc_gl_pow(w, 1 << 31) != 1
    # the reference scaffold's constant is not a 2^32-th root of unity
    assert O.lib().orc_gl_pow(6636018329409361715, 1 << 32) != 1


def test_ct_gs_restatements_match_reference(golden):
    for c in golden["nttct"]:
        out = O.ntt_ct_u32(np.array(c["in"], np.uint32), c["root"], c["mod"])
        assert out.tolist() == c["out"], c["log_n"]
    for c in golden["inttgs"]:
        out = O.intt_gs_u32(np.array(c["in"], np.uint32), c["root"], c["mod"])
        assert out.tolist() == c["out"], c["log_n"]


def test_pwc_convolution_is_cyclic_product(golden):
    for c in golden["pwc"]:
        a = np.array(c["a"], np.int64)
        b = np.array(c["b"], np.int64)
        n = len(a)
        full = O.polymul_u32(a.astype(np.uint32), b.astype(np.uint32), c["mod"]).astype(np.int64)
        cyc = full[:n].copy()
        cyc[: n - 1] += full[n:]
        assert (cyc % c["mod"]).tolist() == c["out"], n


def test_host_input_generator_matches_oracle():
    for p in (65537, 469762049, 2013265921):
        assert np.array_equal(st.uniform_u32_host(5, p, 5000), O.uniform_u32(5, p, 5000))
    assert np.array_equal(st.uniform_gl64_host(9, 5000), O.uniform_u64(9, 5000))


def test_gl_mul_reduction_equals_remainder():
    rng = np.random.default_rng(0)
    vals = [0, 1, 2, O.GL_P - 1, O.GL_P - 2, 2**32, 2**32 - 1, 2**63, 2**64 - 1]
    vals += [int(v) for v in rng.integers(0, 2**63, 200, dtype=np.int64)] + [int(v) * 2 + 1 for v in rng.integers(0, 2**62, 200, dtype=np.int64)]
    L = O.lib()
    for a in vals:
        for b in vals[:40]:
            assert L.orc_gl_mul(a % O.GL_P, b % O.GL_P) == L.orc_gl_mul_slow(a, b) == (a * b) % O.GL_P


def test_dft_point_matches_full_dft():
    for lg in (3, 7, 9):
        n = 1 << lg
        root, p = O.find_params(n, 11)
        x = O.uniform_u32(lg, p, n)
        full = O.dft_u32(x, root, p)
        y = O.uniform_u64(lg, n)
        fg = O.dft_gl64(y, O.gl_root(lg))
        for k in (0, 1, n // 3, n - 1):
            assert O.lib().orc_dft_point_u32(x, n, root, p, k) == full[k]
            assert O.lib().orc_dft_point_gl64(y, n, O.gl_root(lg), k) == fg[k]


@pytest.mark.parametrize("lg", [1, 6, 10])
def test_cyclic_conv_equals_schoolbook(golden, lg):
    """The transform-based cyclic convolution (pwcNtt semantics) against the
    schoolbook product folded modulo x^n - 1, both fields; also against the
    reference's own pwc_convolution vectors."""
    n = 1 << lg
    root, p = O.find_params(n, 11)
    a, b = O.uniform_u32(lg, p, n), O.uniform_u32(lg + 50, p, n)
    full = O.polymul_u32(a, b, p).astype(np.uint64)
    want = full[:n].copy()
    want[: n - 1] = (want[: n - 1] + full[n:]) % p
    assert np.array_equal(O.cyclic_conv_u32(a, b, root, p), want.astype(np.uint32))
    x, y = O.uniform_u64(lg, n), O.uniform_u64(lg + 50, n)
    fg = O.polymul_gl64(x, y)
    wg = fg[:n].copy()
    for i in range(n - 1):
        wg[i] = (int(wg[i]) + int(fg[n + i])) % O.GL_P
    assert np.array_equal(O.cyclic_conv_gl64(x, y), wg)
    for c in golden["pwc"]:
        got = O.cyclic_conv_u32(np.array(c["a"], np.uint32), np.array(c["b"], np.uint32), c["root"], c["mod"])
        assert got.tolist() == c["out"]
