"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle and
the reference's own vectors. Bit-exact everywhere (integer arithmetic).

Cases follow the reference suite (src/tests/cuda/ntt/st_ntt_test.cu:51-97):
util::Rng(42) inputs in [0,9], n = 2^2..2^20 x batches {1,2,5,10}, and the
suite's skipped 2^21..2^26 range; plus uniform residues in [0,p) for both
fields, schoolbook DFT at small n, round trips and linearity at full size.
"""

import hashlib

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).astype("<i4").tobytes()).hexdigest()


def dev32(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32).copy()).cuda()


def host32(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


def dev64(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64).copy()).cuda()


def host64(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint64)


@pytest.fixture(scope="module")
def ref_stream():
    return O.ref_rng_vector(10 << 20)


# --------------------------------------------------------------- 32-bit field
def test_reference_suite_exact(ctx, golden, ref_stream):
    """GPU == oracle (exact field) on every reference-suite case; for n <= 2^13
    also == the unmodified reference output."""
    for case in golden["stockham"]:
        lg, b = case["log_n"], case["batch"]
        if lg > 20:
            continue
        n = 1 << lg
        x = ref_stream[: n * b].astype(np.uint32)
        d = dev32(x)
        ctx.ntt_u32(d, lg, b, case["mod"], case["root"])
        got = host32(d)
        want = O.ntt_u32(x, case["root"], case["mod"], batch=b)
        assert np.array_equal(got, want), (lg, b)
        if lg <= 13:
            assert sha(got.view(np.int32)) == case["sha256"], (lg, b)


def test_reference_suite_ref_wrap(ctx, golden, ref_stream):
    """STNTT_FLAG_REF_WRAP reproduces the reference bit for bit at every n,
    including the suite's skipped 2^21..2^26 range."""
    big = O.ref_rng_vector(1 << 26)
    for case in golden["stockham"]:
        lg, b = case["log_n"], case["batch"]
        n = 1 << lg
        src = ref_stream if n * b <= ref_stream.size else big
        d = dev32(src[: n * b].astype(np.uint32))
        ctx.ntt_u32(d, lg, b, case["mod"], case["root"], ref_wrap=True)
        assert sha(host32(d).view(np.int32)) == case["sha256"], (lg, b)


def test_host_api_mirrors_nttStockham(golden, ref_stream, stntt_lib):
    """st.nttStockham(int32 host array, size, root, mod, batches) in place,
    as src/ntt/ntt_cpu.h:8-9."""
    for case in golden["stockham"]:
        lg, b = case["log_n"], case["batch"]
        if lg > 16:
            continue
        v = ref_stream[: (1 << lg) * b].copy()
        st.nttStockham(v, 1 << lg, case["root"], case["mod"], b, ref_wrap=True)
        assert sha(v) == case["sha256"], (lg, b)
        if lg <= 13:
            w = ref_stream[: (1 << lg) * b].copy()
            st.nttStockham(w, 1 << lg, case["root"], case["mod"], b)
            assert sha(w) == case["sha256"], (lg, b)
    with pytest.raises(st.StnttError, match="must be a power of 2"):
        st.nttStockham(np.zeros(12, np.int32), 12, 1, 13)


@pytest.mark.parametrize("lg", list(range(0, 23)))
def test_u32_uniform_vs_oracle(ctx, lg):
    p, root = st.params_u32(lg)
    b = max(1, (1 << 16) >> lg)
    x = O.uniform_u32(100 + lg, p, b << lg)
    d = dev32(x)
    ctx.ntt_u32(d, lg, b, p, root)
    f = host32(d)
    assert np.array_equal(f, O.ntt_u32(x, root, p, batch=b)), lg
    ctx.ntt_u32(d, lg, b, p, root, inverse=True)
    assert np.array_equal(host32(d), x), lg


@pytest.mark.parametrize("lg", [1, 4, 7, 10])
def test_u32_schoolbook(ctx, lg):
    p, root = st.params_u32(lg)
    x = O.uniform_u32(7 + lg, p, 1 << lg)
    d = dev32(x)
    ctx.ntt_u32(d, lg, 1, p, root)
    assert np.array_equal(host32(d), O.dft_u32(x, root, p))


def test_u32_inverse_vs_oracle(ctx):
    for lg in (3, 9, 13, 14, 19):
        p, root = st.params_u32(lg)
        x = O.uniform_u32(55, p, 2 << lg)
        d = dev32(x)
        ctx.ntt_u32(d, lg, 2, p, root, inverse=True)
        assert np.array_equal(host32(d), O.ntt_u32(x, root, p, inverse=True, batch=2)), lg


def _dft_at(x, w, k, p):
    """X[k] = sum_j x_j w^(jk) mod p for one k (vectorised, p < 2^32)."""
    n = x.size
    B = 1 << ((n.bit_length() - 1 + 1) // 2)
    wk = pow(w, k, p)
    lo = np.empty(B, np.uint64)
    acc = 1
    for i in range(B):
        lo[i] = acc
        acc = acc * wk % p
    hi = np.empty(n // B, np.uint64)
    step = pow(wk, B, p)
    acc = 1
    for i in range(n // B):
        hi[i] = acc
        acc = acc * step % p
    pw = (hi[:, None] * lo[None, :]) % np.uint64(p)
    return int(((x.astype(np.uint64).reshape(-1, B) * pw) % np.uint64(p)).sum() % p)


@pytest.mark.parametrize("lg", [24, 26])
def test_u32_full_size(ctx, lg):
    """u32 2^24 and 2^26 (the large-transform sizes, exact field): forward and
    inverse element for element against the oracle, plus spot DFT values,
    linearity and the round trip."""
    p, root = st.params_u32(lg)
    n = 1 << lg
    x = O.uniform_u32(31, p, n)
    d = dev32(x)
    ctx.ntt_u32(d, lg, 1, p, root)
    f = host32(d)
    assert np.array_equal(f, O.ntt_u32(x, root, p))
    di = dev32(x)
    ctx.ntt_u32(di, lg, 1, p, root, inverse=True)
    assert np.array_equal(host32(di), O.ntt_u32(x, root, p, inverse=True))
    del di
    for k in (0, 1, 12345, n - 1):
        assert int(f[k]) == _dft_at(x, root, k, p), k
    y = O.uniform_u32(32, p, n)
    dy = dev32(y)
    ctx.ntt_u32(dy, lg, 1, p, root)
    s = dev32((x.astype(np.uint64) + y) % p)
    ctx.ntt_u32(s, lg, 1, p, root)
    assert np.array_equal(host32(s), ((f.astype(np.uint64) + host32(dy)) % p).astype(np.uint32))
    ctx.ntt_u32(d, lg, 1, p, root, inverse=True)
    assert np.array_equal(host32(d), x)


def test_u32_partial_steps(ctx):
    """The nsteps hook (ntt_cpu.h:8): first k radix-2 stages, exact and wrap."""
    for lg in (5, 11, 16):
        p, root = st.params_u32(lg)
        x = O.uniform_u32(3, p, 1 << lg)
        for k in (0, 1, lg // 2, lg):
            d = dev32(x)
            ctx.ntt_u32_steps(d, lg, 1, p, root, k)
            want = x.copy()
            O.lib().orc_ntt_u32(want, 1 << lg, root, p, k)
            assert np.array_equal(host32(d), want), (lg, k)
            d = dev32(x)
            ctx.ntt_u32_steps(d, lg, 1, p, root, k, ref_wrap=True)
            w2 = O.ntt_ref_wrap(x.view(np.int32), root, p, nsteps=k)
            assert np.array_equal(host32(d).view(np.int32), w2), (lg, k)


# --------------------------------------------------------------- Goldilocks
@pytest.mark.parametrize("lg", list(range(0, 23)))
def test_gl64_vs_oracle(ctx, lg):
    b = max(1, (1 << 14) >> lg)
    x = O.uniform_u64(500 + lg, b << lg)
    d = dev64(x)
    ctx.ntt_gl64(d, lg, b)
    f = host64(d)
    assert np.array_equal(f, O.ntt_gl64(x, batch=b)), lg
    ctx.ntt_gl64(d, lg, b, inverse=True)
    assert np.array_equal(host64(d), x), lg


@pytest.mark.parametrize("lg", [1, 5, 8, 10])
def test_gl64_schoolbook(ctx, lg):
    x = O.uniform_u64(77 + lg, 1 << lg)
    d = dev64(x)
    ctx.ntt_gl64(d, lg)
    assert np.array_equal(host64(d), O.dft_gl64(x, O.gl_root(lg)))


def test_gl64_inverse_vs_oracle(ctx):
    for lg in (2, 12, 13, 17, 20):
        x = O.uniform_u64(66, 3 << lg)
        d = dev64(x)
        ctx.ntt_gl64(d, lg, 3, inverse=True)
        assert np.array_equal(host64(d), O.ntt_gl64(x, inverse=True, batch=3)), lg


def test_gl64_2e24(ctx):
    """The headline size: Goldilocks 2^24, forward and inverse vs the oracle,
    round trip."""
    lg = 24
    x = O.uniform_u64(2024, 1 << lg)
    d = dev64(x)
    ctx.ntt_gl64(d, lg)
    f = host64(d)
    assert np.array_equal(f, O.ntt_gl64(x, threads=1))
    di = dev64(x)
    ctx.ntt_gl64(di, lg, inverse=True)
    assert np.array_equal(host64(di), O.ntt_gl64(x, inverse=True))
    del di
    ctx.ntt_gl64(d, lg, inverse=True)
    assert np.array_equal(host64(d), x)


def test_gl64_out_of_place(ctx):
    for lg in (6, 15):
        x = O.uniform_u64(4, 1 << lg)
        src = dev64(x)
        dst = torch.zeros_like(src)
        ctx.ntt_gl64_oop(src, dst, lg)
        assert np.array_equal(host64(src), x)
        assert np.array_equal(host64(dst), O.ntt_gl64(x))


# --------------------------------------------------------------- polymul
@pytest.mark.parametrize("lg", [1, 6, 12])
def test_polymul_u32_vs_schoolbook(ctx, lg):
    p, root = st.params_u32(lg)
    n = 1 << lg
    h = max(1, n // 2)
    a = np.zeros(n, np.uint32)
    b = np.zeros(n, np.uint32)
    a[:h] = O.uniform_u32(1, p, h)
    b[:h] = O.uniform_u32(2, p, h)
    da, db = dev32(a), dev32(b)
    out = torch.empty_like(da)
    ctx.polymul_u32(da, db, out, lg, p, root)
    want = O.polymul_u32(a[:h], b[:h], p)
    got = host32(out)
    assert np.array_equal(got[: want.size], want)
    assert not got[want.size:].any()


@pytest.mark.parametrize("lg", [1, 6, 12])
def test_polymul_gl64_vs_schoolbook(ctx, lg):
    n = 1 << lg
    h = max(1, n // 2)
    a = np.zeros(n, np.uint64)
    b = np.zeros(n, np.uint64)
    a[:h] = O.uniform_u64(3, h)
    b[:h] = O.uniform_u64(4, h)
    da, db = dev64(a), dev64(b)
    ctx.polymul_gl64(da, db, da, lg)  # output aliases an input
    want = O.polymul_gl64(a[:h], b[:h])
    got = host64(da)
    assert np.array_equal(got[: want.size], want)


def test_pwc_convolution_semantics(ctx, golden):
    """pwc_convolution (ntt_cpu.cpp:180-193): cyclic product with p >= max^2*len+1."""
    for c in golden["pwc"]:
        n = len(c["a"])
        lg = n.bit_length() - 1
        root, mod = st.findParams(n, max(max(c["a"]), max(c["b"])) ** 2 * n + 1)
        assert (root, mod) == (c["root"], c["mod"])
        da, db = dev32(np.array(c["a"], np.uint32)), dev32(np.array(c["b"], np.uint32))
        out = torch.empty_like(da)
        ctx.polymul_u32(da, db, out, lg, mod, root)
        assert host32(out).tolist() == c["out"], n


# --------------------------------------------------------------- batches, inputs, errors
def test_batch_jobs_match_single_calls(ctx):
    rng = np.random.default_rng(5)
    jobs, bufs, want = [], [], []
    for i in range(24):
        lg = int(rng.integers(1, 16))
        inv = i % 2
        if i % 3 == 0:
            p, root = st.params_u32(lg)
            x = O.uniform_u32(i, p, 1 << lg)
            d = dev32(x)
            jobs.append(st.Job(st.FIELD_U32, lg, inv, p, root, 0, d.data_ptr()))
            want.append(O.ntt_u32(x, root, p, inverse=bool(inv)))
        else:
            x = O.uniform_u64(i, 1 << lg)
            d = dev64(x)
            jobs.append(st.Job(st.FIELD_GL64, lg, inv, 0, 0, 0, d.data_ptr()))
            want.append(O.ntt_gl64(x, inverse=bool(inv)))
        bufs.append(d)
    ctx.ntt_batch(jobs)
    torch.cuda.synchronize()
    for d, w in zip(bufs, want):
        got = host32(d) if d.dtype == torch.int32 else host64(d)
        assert np.array_equal(got, w)


def test_device_input_generator_matches_host(stntt_lib):
    t = torch.empty(70000, dtype=torch.int32, device="cuda")
    st.fill_uniform_u32(t, 11, 469762049)
    assert np.array_equal(host32(t), O.uniform_u32(11, 469762049, 70000))
    g = torch.empty(70000, dtype=torch.int64, device="cuda")
    st.fill_uniform_gl64(g, 12)
    assert np.array_equal(host64(g), O.uniform_u64(12, 70000))


def test_argument_errors(ctx):
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(st.StnttError, match="EINVAL"):
        ctx.ntt_u32(d, 4, 1, 65537, 2)  # 2 is not a primitive 16th root mod 65537
    with pytest.raises(st.StnttError, match="EINVAL"):
        ctx.ntt_u32(d, 4, 1, 65536, 3)
    with pytest.raises(st.StnttError, match="EUNSUPPORTED"):
        ctx.ntt_u32(d, 28, 1, 65537, 3)
    with pytest.raises(st.StnttError, match="EINVAL"):
        ctx.ntt_u32(d, 4, 1, 65537, 3, inverse=True, ref_wrap=True)
    g = torch.zeros(16, dtype=torch.int64, device="cuda")
    with pytest.raises(st.StnttError, match="EUNSUPPORTED"):
        ctx.ntt_gl64(g, 33)
    # state stays usable
    p, root = st.params_u32(4)
    ctx.ntt_u32(d, 4, 1, p, root)
    assert not host32(d).any()


@pytest.mark.parametrize("lg", [3, 10, 14, 20])
def test_u32_primes_above_2e30(ctx, lg):
    """Primes in [2^30, 2^31) take the strict-reduction kernels (the lazy ones
    need 4p < 2^32)."""
    root, p = st.findParams(1 << lg, 1 << 30)
    assert (1 << 30) <= p < (1 << 31)
    x = O.uniform_u32(9 + lg, p, 2 << lg)
    d = dev32(x)
    ctx.ntt_u32(d, lg, 2, p, root)
    assert np.array_equal(host32(d), O.ntt_u32(x, root, p, batch=2))
    ctx.ntt_u32(d, lg, 2, p, root, inverse=True)
    assert np.array_equal(host32(d), x)
    a = np.zeros(1 << lg, np.uint32)
    b = np.zeros(1 << lg, np.uint32)
    h = max(1, (1 << lg) // 2)
    a[:h], b[:h] = O.uniform_u32(1, p, h), O.uniform_u32(2, p, h)
    out = torch.empty(1 << lg, dtype=torch.int32, device="cuda")
    ctx.polymul_u32(dev32(a), dev32(b), out, lg, p, root)
    if lg <= 10:
        want = O.polymul_u32(a[:h], b[:h], p)
        assert np.array_equal(host32(out)[: want.size], want)



@pytest.mark.parametrize("lg", [10, 14, 20, 22])
def test_u32_primes_between_2e29_and_2e30(ctx, lg):
    """Primes in [2^29, 2^30) keep the lazy field but not the vector-lines
    steps, whose bound-tracked DFTs need 8p < 2^32: their plans fall back to
    the plain tile. Single and batched transforms against the oracle, and the
    round trip."""
    root, p = st.findParams(1 << lg, 1 << 29)
    assert (1 << 29) <= p < (1 << 30)
    for batch in (1, 2):
        x = O.uniform_u32(31 + lg + batch, p, batch << lg)
        d = dev32(x)
        ctx.ntt_u32(d, lg, batch, p, root)
        assert np.array_equal(host32(d), O.ntt_u32(x, root, p, batch=batch)), (lg, batch)
        ctx.ntt_u32(d, lg, batch, p, root, inverse=True)
        assert np.array_equal(host32(d), x), (lg, batch)


def _gl_add(a, b):
    """(a + b) mod p for canonical uint64 arrays, with wrap-around arithmetic."""
    with np.errstate(over="ignore"):
        s = a + b
        wrap = (s < a) | (s >= np.uint64(O.GL_P))
        return np.where(wrap, s - np.uint64(O.GL_P), s)


def test_largest_sizes_three_pass(ctx):
    """Goldilocks 2^26 and the 32-bit prime 2^27 (p = 2013265921 >= 2^30: the
    strict-reduction kernels), both three HBM passes: spot DFT values from the
    oracle, linearity, round trip."""
    for field, lg in (("gl64", 26), ("u32", 27)):
        n = 1 << lg
        if field == "gl64":
            x, y = O.uniform_u64(71, n), O.uniform_u64(72, n)
            d, dy = dev64(x), dev64(y)
            ctx.ntt_gl64(d, lg)
            ctx.ntt_gl64(dy, lg)
            f, fy = host64(d), host64(dy)
            root = O.gl_root(lg)
            for k in (0, 1, 777, n - 1):
                assert int(f[k]) == O.lib().orc_dft_point_gl64(x, n, root, k), (field, k)
            # linearity on the transform of x + y
            ds = dev64(_gl_add(x, y))
            ctx.ntt_gl64(ds, lg)
            assert np.array_equal(host64(ds), _gl_add(f, fy))
            ctx.ntt_gl64(d, lg, inverse=True)
            assert np.array_equal(host64(d), x)
        else:
            p, root = st.params_u32(lg)
            assert p == 2013265921
            x = O.uniform_u32(73, p, n)
            d = dev32(x)
            ctx.ntt_u32(d, lg, 1, p, root)
            f = host32(d)
            for k in (0, 1, 777, n - 1):
                assert int(f[k]) == O.lib().orc_dft_point_u32(x, n, root, p, k), (field, k)
            ctx.ntt_u32(d, lg, 1, p, root, inverse=True)
            assert np.array_equal(host32(d), x)


def test_empty_and_null_arguments(ctx):
    p, root = st.params_u32(10)
    assert st.lib().stntt_ntt_u32(ctx.handle, None, 10, 0, p, root, 0, 0, None) == 0  # empty batch: no-op
    assert st.lib().stntt_ntt_gl64(ctx.handle, None, 10, 0, 0, None) == 0
    assert st.lib().stntt_ntt_u32(ctx.handle, None, 10, 1, p, root, 0, 0, None) == 1  # null data: EINVAL
    assert st.lib().stntt_ntt_gl64(ctx.handle, None, 10, 1, 0, None) == 1
    assert st.lib().stntt_ntt_batch(ctx.handle, None, 0, None) == 0


def test_single_transforms_in_a_cuda_graph(ctx):
    """The device calls are capturable: forward + inverse captured once per
    size on a side stream (after a warm-up call on it builds the plan and its
    workspace), replayed; results equal the oracle and the round trip."""
    s = torch.cuda.Stream()
    for field, lg in (("u32", 16), ("gl64", 20), ("u32", 13)):
        n = 1 << lg
        if field == "gl64":
            x = O.uniform_u64(90 + lg, n)
            d = dev64(x)
            fwd = lambda: ctx.ntt_gl64(d, lg, stream=s.cuda_stream)  # noqa: E731
            inv = lambda: ctx.ntt_gl64(d, lg, inverse=True, stream=s.cuda_stream)  # noqa: E731
            want, host = O.ntt_gl64(x), host64
        else:
            p, root = st.params_u32(lg)
            x = O.uniform_u32(90 + lg, p, n)
            d = dev32(x)
            fwd = lambda: ctx.ntt_u32(d, lg, 1, p, root, stream=s.cuda_stream)  # noqa: E731
            inv = lambda: ctx.ntt_u32(d, lg, 1, p, root, inverse=True, stream=s.cuda_stream)  # noqa: E731
            want, host = O.ntt_u32(x, root, p), host32
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            fwd()
            inv()
        torch.cuda.synchronize()
        gf, gi = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
        with torch.cuda.graph(gf, stream=s, capture_error_mode="relaxed"):
            fwd()
        with torch.cuda.graph(gi, stream=s, capture_error_mode="relaxed"):
            inv()
        with torch.cuda.stream(s):
            gf.replay()
        assert np.array_equal(host(d), want), (field, lg)
        with torch.cuda.stream(s):
            gi.replay()
            for _ in range(3):
                gf.replay()
                gi.replay()
        assert np.array_equal(host(d), x), (field, lg)


def test_small_call_plans(ctx):
    """stntt_set_plan_small: a separate shape for calls of fewer than 2^22
    elements; single transforms take it, a 2^22-element batch takes the main
    plan, and both are bit-exact."""
    try:
        for field, lg in (("gl64", 16), ("u32", 16)):
            fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
            ctx.set_plan(fid, lg, [6, 10], [16, 16], [8, 2], small=True)
            ctx.set_plan(fid, lg, [9, 7], [16, 16], [4, 16])
            for batch in (1, 64):
                n = batch << lg
                if field == "gl64":
                    x = O.uniform_u64(300 + batch, n)
                    d = dev64(x)
                    ctx.ntt_gl64(d, lg, batch)
                    assert np.array_equal(host64(d), O.ntt_gl64(x, batch=batch, threads=8)), (field, batch)
                    ctx.ntt_gl64(d, lg, batch, inverse=True)
                    assert np.array_equal(host64(d), x)
                else:
                    p, root = st.params_u32(lg)
                    x = O.uniform_u32(300 + batch, p, n)
                    d = dev32(x)
                    ctx.ntt_u32(d, lg, batch, p, root)
                    assert np.array_equal(host32(d), O.ntt_u32(x, root, p, batch=batch, threads=8)), (field, batch)
                    ctx.ntt_u32(d, lg, batch, p, root, inverse=True)
                    assert np.array_equal(host32(d), x)
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


@pytest.mark.parametrize("field,lg", [("u32", 14), ("u32", 15), ("u32", 16), ("gl64", 14), ("gl64", 15)])
def test_cluster_path(ctx, field, lg):
    """Small two-pass calls run as one thread-block-cluster launch (both passes
    exchanging through distributed shared memory): batches of 1, 3 and 8,
    forward and inverse, in place and out of place, equal the oracle."""
    n = 1 << lg
    for batch in (1, 3, 8):
        if field == "gl64":
            x = O.uniform_u64(500 + lg + batch, batch * n)
            want = O.ntt_gl64(x, batch=batch, threads=8)
            d = dev64(x)
            o = torch.empty_like(d)
            ctx.ntt_gl64_oop(d, o, lg, batch)
            assert np.array_equal(host64(o), want), (lg, batch)
            ctx.ntt_gl64(d, lg, batch)
            assert np.array_equal(host64(d), want), (lg, batch)
            ctx.ntt_gl64(d, lg, batch, inverse=True)
            assert np.array_equal(host64(d), x), (lg, batch)
        else:
            p, root = st.params_u32(lg)
            x = O.uniform_u32(500 + lg + batch, p, batch * n)
            want = O.ntt_u32(x, root, p, batch=batch, threads=8)
            d = dev32(x)
            o = torch.empty_like(d)
            ctx.ntt_u32_oop(d, o, lg, batch, p, root)
            assert np.array_equal(host32(o), want), (lg, batch)
            ctx.ntt_u32(d, lg, batch, p, root)
            assert np.array_equal(host32(d), want), (lg, batch)
            ctx.ntt_u32(d, lg, batch, p, root, inverse=True)
            assert np.array_equal(host32(d), x), (lg, batch)


def test_call_info_reports_launches(ctx):
    """stntt_call_info: one launch for a small call on the cluster path, the
    plan's pass count otherwise."""
    p16, r16 = st.params_u32(16)
    assert ctx.call_info(st.FIELD_U32, 16, 1, p16, r16)[0] == 1
    n, logs = ctx.call_info(st.FIELD_U32, 16, 64, p16, r16)  # 2^22 elements: not a small call
    assert n == len(logs) >= 2 and sum(logs) == 16
    n, logs = ctx.call_info(st.FIELD_GL64, 16, 1)  # 512 KiB: one 16-CTA cluster launch where the device has them
    assert n in (1, 2) and len(logs) == 2 and sum(logs) == 16
    n, logs = ctx.call_info(st.FIELD_GL64, 17, 1)  # 1 MiB: beyond the cluster path
    assert n == len(logs) == 2 and sum(logs) == 17
    n, logs = ctx.call_info(st.FIELD_GL64, 24, 1)
    assert n == len(logs) and sum(logs) == 24


@pytest.mark.parametrize("field,lg,logs,cols", [
    ("gl64", 14, [7, 7], [4, 8]), ("gl64", 18, [9, 9], [2, 4]), ("gl64", 20, [10, 10], [4, 2]),
    ("gl64", 21, [7, 7, 7], [8, 8, 2]), ("u32", 16, [8, 8], [8, 8]), ("u32", 22, [11, 11], [2, 2])])
def test_eight_element_tiles(ctx, field, lg, logs, cols):
    """Plans with 8 elements per thread (radix-8 steps, twice the threads per
    tile) are bit-exact, forward, inverse and in a polynomial product whose
    inverse falls back to a separate pointwise product."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    try:
        for small in (False, True):
            ctx.set_plan(fid, lg, logs, [8] * len(logs), cols, small=small)
        for batch in (1, 3):
            n = batch << lg
            if field == "gl64":
                x = O.uniform_u64(600 + lg + batch, n)
                d = dev64(x)
                ctx.ntt_gl64(d, lg, batch)
                assert np.array_equal(host64(d), O.ntt_gl64(x, batch=batch, threads=8)), (lg, batch)
                ctx.ntt_gl64(d, lg, batch, inverse=True)
                assert np.array_equal(host64(d), x), (lg, batch)
            else:
                p, root = st.params_u32(lg)
                x = O.uniform_u32(600 + lg + batch, p, n)
                d = dev32(x)
                ctx.ntt_u32(d, lg, batch, p, root)
                assert np.array_equal(host32(d), O.ntt_u32(x, root, p, batch=batch, threads=8)), (lg, batch)
                ctx.ntt_u32(d, lg, batch, p, root, inverse=True)
                assert np.array_equal(host32(d), x), (lg, batch)
        if field == "gl64" and lg <= 14:
            n = 1 << lg
            h = n // 2
            a = np.zeros(n, np.uint64)
            b = np.zeros(n, np.uint64)
            a[:h] = O.uniform_u64(610, h)
            b[:h] = O.uniform_u64(611, h)
            out = torch.empty(n, dtype=torch.int64, device="cuda")
            ctx.polymul_gl64(dev64(a), dev64(b), out, lg)
            want = O.polymul_gl64(a[:h], b[:h])
            assert np.array_equal(host64(out)[: want.size], want)
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


@pytest.mark.parametrize("field,lg,logs", [("u32", 16, [8, 8]), ("u32", 17, [8, 9]), ("gl64", 16, [8, 8]),
                                           ("gl64", 16, [9, 7])])
def test_cluster_path_eight_elements(ctx, field, lg, logs):
    """Small-call plans with 8 elements per thread run the cluster path with
    twice the threads per CTA where its shape allows it; bit-exact either way."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    try:
        ctx.set_plan(fid, lg, logs, [8, 8], small=True)
        p, root = (0, 0) if field == "gl64" else st.params_u32(lg)
        launches, _ = ctx.call_info(fid, lg, 1, p, root)
        assert launches in (1, 2)
        for batch in (1, 3):
            n = batch << lg
            if field == "gl64":
                x = O.uniform_u64(700 + lg + batch, n)
                d = dev64(x)
                ctx.ntt_gl64(d, lg, batch)
                assert np.array_equal(host64(d), O.ntt_gl64(x, batch=batch, threads=8)), (lg, batch)
                ctx.ntt_gl64(d, lg, batch, inverse=True)
                assert np.array_equal(host64(d), x), (lg, batch)
            else:
                x = O.uniform_u32(700 + lg + batch, p, n)
                d = dev32(x)
                ctx.ntt_u32(d, lg, batch, p, root)
                assert np.array_equal(host32(d), O.ntt_u32(x, root, p, batch=batch, threads=8)), (lg, batch)
                ctx.ntt_u32(d, lg, batch, p, root, inverse=True)
                assert np.array_equal(host32(d), x), (lg, batch)
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


def test_stream_workspaces_release_and_cap(ctx):
    """Per-stream scratch: stntt_release_stream frees a stream's buffer, and a
    context keeps at most 64 of them (least recently used freed first)."""
    lg = 18  # two HBM passes (no one-launch cluster at this size): a 2^18 * 8-byte workspace per stream
    ws = (1 << lg) * 8
    x = O.uniform_u64(3, 1 << lg)
    want = O.ntt_gl64(x)
    d = dev64(x)
    ctx.ntt_gl64(d, lg)  # plan and tables for this size
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream() for _ in range(70)]
    base = ctx.mem_usage()
    for i, s in enumerate(streams):
        di = dev64(x)
        ctx.ntt_gl64(di, lg, stream=s)
        s.synchronize()
        assert np.array_equal(host64(di), want), i
    grown = ctx.mem_usage() - base
    assert 0 < grown <= 64 * ws
    for s in streams:
        ctx.release_stream(s)
    assert ctx.mem_usage() <= base
    # still usable afterwards on a released stream
    di = dev64(x)
    ctx.ntt_gl64(di, lg, stream=streams[0])
    streams[0].synchronize()
    assert np.array_equal(host64(di), want)
    ctx.release_stream(streams[0])


def test_host_call_reports_kernel_time(ctx):
    """stntt_last_kernel_ms: the device time of the last host-buffer call (what
    the reference's autoNtt returns)."""
    lg = 16
    p, root = st.params_u32(lg)
    v = O.ref_rng_vector(1 << lg)
    ctx.ntt_stockham_host(v, 1 << lg, root, p, ref_wrap=True)
    assert ctx.last_kernel_ms() > 0.0
    y = O.uniform_u64(5, 1 << 20)
    ctx.ntt_gl64_host(y, 20)
    assert ctx.last_kernel_ms() > 0.0


VEC = st.PASS_VEC


@pytest.mark.parametrize("field,lg,logs,batch,cols", [
    ("gl64", 16, [8, 8], 64, 16),      # column pass with a full four-step table, row pass; 8 line groups
    ("gl64", 22, [7, 7, 8], 1, 8),     # two-level four-step twiddle, full table, row; 4 line groups
    ("gl64", 20, [10, 10], 4, 16),
    ("gl64", 18, [9, 9], 16, 8),
    ("u32", 16, [8, 8], 64, 32),
    ("u32", 22, [7, 7, 8], 1, 16),
    ("u32", 20, [10, 10], 4, 32),
    ("u32", 18, [9, 9], 16, 16),
    ("gl64", 22, [11, 11], 1, 4),      # wide two-pass tiles, 2 line groups (padded shared memory)
    ("gl64", 23, [11, 12], 1, 4),
    ("u32", 22, [11, 11], 1, 16),      # 4 line groups of 2^11 points
    ("u32", 23, [12, 11], 1, 8),
    ("gl64", 20, [9, 11], 2, 2),       # one line group of 2^11 points (the narrowest, padded)
    ("u32", 21, [10, 11], 1, 4),
])
def test_vector_lines_build(ctx, field, lg, logs, batch, cols):
    """STNTT_PASS_VEC: every pass in the vector-lines build (V adjacent lines
    per thread, 16-byte accesses), forward and inverse, against the oracle;
    an unaligned output falls back to the plain build with the same result."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    k = len(logs)
    try:
        ctx.clear_plans()  # without the packaged small-call shapes, calls under 2^22 elements take this plan too
        ctx.set_plan(fid, lg, logs, elems=[16 | VEC] * k, cols=[cols] * k)
        n = 1 << lg
        if field == "gl64":
            x = O.uniform_u64(900 + lg, batch * n)
            for inv in (False, True):
                d = dev64(x)
                ctx.ntt_gl64(d, lg, batch, inverse=inv)
                assert np.array_equal(host64(d), O.ntt_gl64(x, inverse=inv, batch=batch, threads=8)), inv
            src = dev64(x)
            big = torch.zeros(batch * n + 1, dtype=torch.int64, device="cuda")
            ctx.ntt_gl64_oop(src, big[1:], lg, batch)
            assert np.array_equal(host64(big[1:]), O.ntt_gl64(x, batch=batch, threads=8))
        else:
            p, root = st.params_u32(lg)
            x = O.uniform_u32(900 + lg, p, batch * n)
            for inv in (False, True):
                d = dev32(x)
                ctx.ntt_u32(d, lg, batch, p, root, inverse=inv)
                assert np.array_equal(host32(d), O.ntt_u32(x, root, p, inverse=inv, batch=batch, threads=8)), inv
            src = dev32(x)
            big = torch.zeros(batch * n + 1, dtype=torch.int32, device="cuda")
            ctx.ntt_u32_oop(src, big[1:], lg, batch, p, root)
            assert np.array_equal(host32(big[1:]), O.ntt_u32(x, root, p, batch=batch, threads=8))
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


@pytest.mark.parametrize("field,lg,logs,cols", [("gl64", 24, [8, 8, 8], 16), ("u32", 26, [8, 9, 9], 32),
                                                ("gl64", 24, [8, 8, 8], 8), ("u32", 26, [8, 9, 9], 16),
                                                ("gl64", 24, [12, 12], 4), ("u32", 24, [12, 12], 8)])
def test_vector_lines_build_full_size(ctx, field, lg, logs, cols):
    """The large transforms in the vector-lines build equal the plain build
    (which the oracle pins at these sizes) bit for bit, both directions."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    n = 1 << lg
    p, root = (0, 0) if field == "gl64" else st.params_u32(lg)
    if field == "gl64":
        x = torch.empty(n, dtype=torch.int64, device="cuda")
        st.fill_uniform_gl64(x, 5)
        run = lambda t, inv: ctx.ntt_gl64(t, lg, 1, inverse=inv)  # noqa: E731
    else:
        x = torch.empty(n, dtype=torch.int32, device="cuda")
        st.fill_uniform_u32(x, 5, p)
        run = lambda t, inv: ctx.ntt_u32(t, lg, 1, p, root, inverse=inv)  # noqa: E731
    try:
        want = {}
        ctx.set_plan(fid, lg, logs)
        for inv in (False, True):
            t = x.clone()
            run(t, inv)
            want[inv] = t
        ctx.set_plan(fid, lg, logs, elems=[16 | VEC] * len(logs), cols=[cols] * len(logs))
        for inv in (False, True):
            t = x.clone()
            run(t, inv)
            torch.cuda.synchronize()
            assert torch.equal(t, want[inv]), inv
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


@pytest.mark.parametrize("field,lg", [("gl64", 18), ("gl64", 19), ("gl64", 20), ("gl64", 21),
                                      ("u32", 18), ("u32", 19), ("u32", 20), ("u32", 21)])
def test_cooperative_two_pass_launch(ctx, field, lg):
    """stntt_set_coop(1): single calls of 2^18..2^21 points run both passes in
    one cooperative launch (grid-wide barrier): one launch per call,
    bit-exact against the oracle in both directions, again after many calls
    on one stream (the barrier words are reused), on a second stream, inside
    a replayed CUDA graph, and equal to the two-launch path (the default)."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    p, root = (0, 0) if field == "gl64" else st.params_u32(lg)
    ctx.set_plan(fid, lg, [lg // 2, lg - lg // 2], elems=[8, 8], small=True)
    ctx.set_coop(1)
    launches, _ = ctx.call_info(fid, lg, 1, p, root)
    assert launches == 1
    n = 1 << lg
    if field == "gl64":
        x = O.uniform_u64(40 + lg, n)
        want = {False: O.ntt_gl64(x), True: O.ntt_gl64(x, inverse=True)}
        mk, get = dev64, host64
        run = lambda t, inv, s=None: ctx.ntt_gl64(t, lg, 1, inverse=inv, stream=s)  # noqa: E731
    else:
        x = O.uniform_u32(40 + lg, p, n)
        want = {False: O.ntt_u32(x, root, p), True: O.ntt_u32(x, root, p, inverse=True)}
        mk, get = dev32, host32
        run = lambda t, inv, s=None: ctx.ntt_u32(t, lg, 1, p, root, inverse=inv, stream=s)  # noqa: E731
    for inv in (False, True):
        d = mk(x)
        run(d, inv)
        assert np.array_equal(get(d), want[inv]), inv
    d = mk(x)
    for _ in range(25):  # forward + inverse, many barrier generations on one stream
        run(d, False)
        run(d, True)
    assert np.array_equal(get(d), x)
    s2 = torch.cuda.Stream()
    d2 = mk(x)
    run(d2, False, s2)
    s2.synchronize()
    assert np.array_equal(get(d2), want[False])
    g = torch.cuda.CUDAGraph()
    d3 = mk(x)
    with torch.cuda.graph(g, stream=s2):
        run(d3, False, s2)
    for _ in range(2):
        d3.copy_(mk(x))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(get(d3), want[False])
    assert ctx.device_status() == 0
    try:
        ctx.set_coop(0)  # the default: two launches
        assert ctx.call_info(fid, lg, 1, p, root)[0] == 2
        d4 = mk(x)
        run(d4, False)
        assert np.array_equal(get(d4), want[False])
    finally:
        ctx.set_coop(0)
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


GL_P = (1 << 64) - (1 << 32) + 1
GL_EDGE = np.array([0, 1, 2, GL_P - 1, GL_P - 2, (1 << 32) - 1, 1 << 32, (1 << 32) + 1, 1 << 63, (1 << 63) - 1,
                    GL_P - (1 << 32), (GL_P - 1) // 2, 0xFFFFFFFF00000000, 0x00000000FFFFFFFF, 0x8000000080000000,
                    0x7FFFFFFF7FFFFFFF], dtype=np.uint64)


@pytest.mark.parametrize("lg,logs,elems,cols", [(16, [8, 8], 8, 8), (16, [8, 8], 16, 16), (22, [7, 8, 7], 8, 8),
                                                (20, [10, 10], 16, 4)])
def test_gl64_edge_values(ctx, lg, logs, elems, cols):
    """Goldilocks passes with shift-only internal twiddles (radix-4/8 with 8
    points per line, radix-16 with 16: every w_16^q = +-2^e) on inputs built
    from limb-boundary residues (0, 1, p - 1, 2^32 - 1, 2^32, 2^63, ...):
    both directions against the oracle, and the tuned plan as well."""
    n = 1 << lg
    rng = np.random.default_rng(lg)
    x = GL_EDGE[rng.integers(0, len(GL_EDGE), n)]
    x[: len(GL_EDGE)] = GL_EDGE
    try:
        for plan in ("tuned", "vec"):
            if plan == "vec":
                ctx.clear_plans()  # the packaged small-call shape would take a single 2^16 / 2^20 call
                ctx.set_plan(st.FIELD_GL64, lg, logs, elems=[elems | VEC] * len(logs), cols=[cols] * len(logs))
            for inv in (False, True):
                d = dev64(x)
                ctx.ntt_gl64(d, lg, 1, inverse=inv)
                assert np.array_equal(host64(d), O.ntt_gl64(x, inverse=inv, threads=8)), (plan, inv)
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


CL = st.PASS_CLUSTER


@pytest.mark.parametrize("field,lg,logs,cols,batch", [
    ("gl64", 22, [11, 11], 8, 1),    # every pass in the cluster build, against the oracle
    ("u32", 22, [11, 11], 16, 1),
    ("gl64", 20, [11, 9], 16, 2),    # cluster column pass, then a vector-lines row pass
    ("u32", 21, [9, 12], 32, 1),     # vector-lines column pass, then a cluster row pass
])
def test_vector_lines_cluster_pass(ctx, field, lg, logs, cols, batch):
    """STNTT_PASS_CLUSTER: passes whose line DFTs are spread over the 8 CTAs
    of a thread-block cluster (distributed shared memory), forward and
    inverse, against the oracle."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    elems = [(8 | VEC | CL) if lg_ >= 11 else (8 | VEC) for lg_ in logs]
    try:
        ctx.clear_plans()  # without the packaged small-call shapes, calls under 2^22 elements take this plan too
        ctx.set_plan(fid, lg, logs, elems=elems, cols=[cols] * len(logs))
        n = 1 << lg
        for inv in (False, True):
            if field == "gl64":
                x = O.uniform_u64(700 + lg, batch * n)
                d = dev64(x)
                ctx.ntt_gl64(d, lg, batch, inverse=inv)
                assert np.array_equal(host64(d), O.ntt_gl64(x, inverse=inv, batch=batch, threads=8)), inv
            else:
                p, root = st.params_u32(lg)
                x = O.uniform_u32(700 + lg, p, batch * n)
                d = dev32(x)
                ctx.ntt_u32(d, lg, batch, p, root, inverse=inv)
                assert np.array_equal(host32(d), O.ntt_u32(x, root, p, inverse=inv, batch=batch, threads=8)), inv
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


@pytest.mark.parametrize("field,lg,logs,cols", [("gl64", 24, [12, 12], 8), ("gl64", 24, [12, 12], 16),
                                                ("u32", 26, [13, 13], 16), ("u32", 26, [13, 13], 32),
                                                ("u32", 24, [12, 12], 16), ("gl64", 25, [12, 13], 8)])
def test_vector_lines_cluster_pass_full_size(ctx, field, lg, logs, cols):
    """Two-pass plans with cluster passes at 2^24..2^26 equal the tuned
    plan (pinned against the oracle at these sizes) bit for bit, both
    directions."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    n = 1 << lg
    p, root = (0, 0) if field == "gl64" else st.params_u32(lg)
    if field == "gl64":
        x = torch.empty(n, dtype=torch.int64, device="cuda")
        st.fill_uniform_gl64(x, 6)
        run = lambda t, inv: ctx.ntt_gl64(t, lg, 1, inverse=inv)  # noqa: E731
    else:
        x = torch.empty(n, dtype=torch.int32, device="cuda")
        st.fill_uniform_u32(x, 6, p)
        run = lambda t, inv: ctx.ntt_u32(t, lg, 1, p, root, inverse=inv)  # noqa: E731
    try:
        want = {}
        for inv in (False, True):
            t = x.clone()
            run(t, inv)
            want[inv] = t
        ctx.set_plan(fid, lg, logs, elems=[8 | VEC | CL] * len(logs), cols=[cols] * len(logs))
        for inv in (False, True):
            t = x.clone()
            run(t, inv)
            torch.cuda.synchronize()
            assert torch.equal(t, want[inv]), inv
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


@pytest.mark.parametrize("field,lg,logs,cols", [("gl64", 20, [11, 9], [2, 8]), ("gl64", 18, [9, 9], [16, 8]),
                                                ("u32", 20, [9, 11], [16, 4]), ("u32", 21, [10, 11], [16, 4])])
def test_vector_lines_four_points_per_line(ctx, field, lg, logs, cols):
    """4 points per line (radix-4 steps, twice the threads): the passes of
    single small transforms, forward and inverse against the oracle."""
    fid = st.FIELD_GL64 if field == "gl64" else st.FIELD_U32
    try:
        ctx.clear_plans()  # without the packaged small-call shapes, single calls take this plan
        ctx.set_plan(fid, lg, logs, elems=[4 | VEC] * len(logs), cols=cols)
        n = 1 << lg
        for inv in (False, True):
            if field == "gl64":
                x = O.uniform_u64(600 + lg, n)
                d = dev64(x)
                ctx.ntt_gl64(d, lg, 1, inverse=inv)
                assert np.array_equal(host64(d), O.ntt_gl64(x, inverse=inv, threads=8)), inv
            else:
                p, root = st.params_u32(lg)
                x = O.uniform_u32(600 + lg, p, n)
                d = dev32(x)
                ctx.ntt_u32(d, lg, 1, p, root, inverse=inv)
                assert np.array_equal(host32(d), O.ntt_u32(x, root, p, inverse=inv, threads=8)), inv
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)
