"""The serving loop: mixed NTT and polynomial-product requests arriving over
time, overlapped on one GPU. Each result must be bit-identical to the same
request run alone, and correct against the oracle (products against
schoolbook multiplication at n <= 2^12)."""

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _pinned(n, dtype):
    t = torch.zeros(n, dtype=dtype, pin_memory=True)
    return t, t.numpy()


def _make_trace(seed, count, lo, hi, rate):
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    reqs, keep, expect = [], [], []
    for i in range(count):
        lg = int(rng.integers(lo, hi + 1))
        n = 1 << lg
        gl = bool(rng.integers(0, 2))
        poly = rng.random() < 0.3
        dt = torch.int64 if gl else torch.int32
        ta, a = _pinned(n, dt)
        tb, b = _pinned(n, dt)
        to, out = _pinned(n, dt)
        view = np.uint64 if gl else np.uint32
        if gl:
            p = root = 0
            src = lambda s, k: O.uniform_u64(s, k)  # noqa: E731
        else:
            p, root = st.params_u32(lg)
            src = lambda s, k: O.uniform_u32(s, p, k)  # noqa: E731
        h = max(1, n // 2)
        if poly:
            a.view(view)[:h] = src(1000 + i, h)
            b.view(view)[:h] = src(5000 + i, h)
            want = (O.polymul_gl64 if gl else (lambda x, y: O.polymul_u32(x, y, p)))(
                a.view(view)[:h].copy(), b.view(view)[:h].copy()) if n <= (1 << 12) else None
        else:
            a.view(view)[:] = src(1000 + i, n)
            want = None
        d = int(rng.integers(0, 2))
        reqs.append(st.Request(st.REQ_POLYMUL if poly else st.REQ_NTT, st.FIELD_GL64 if gl else st.FIELD_U32, lg,
                               d, p, root, i, ta.data_ptr(), tb.data_ptr(), to.data_ptr()))
        keep.append((ta, tb, to, a, b, out, view, gl, poly, lg, d, p, root))
        expect.append(want)
    return reqs, list(arrivals), keep, expect


def test_serving_results_match_alone_and_oracle(ctx):
    sv = st.Server(ctx, streams=8, max_log_n=16)
    try:
        reqs, arr, keep, expect = _make_trace(1, 160, 4, 14, rate=50000.0)
        comps = sv.run_trace(reqs, arr)
        assert all(c.status == 0 for c in comps)
        assert all(c.done_s >= c.start_s >= c.submit_s - 1e-6 for c in comps)
        mix = [k[5].copy() for k in keep]
        for i, (ta, tb, to, a, b, out, view, gl, poly, lg, d, p, root) in enumerate(keep):
            res = mix[i].view(view)
            # oracle
            if poly:
                if expect[i] is not None:
                    want = expect[i]
                    assert np.array_equal(res[: want.size], want), i
            else:
                x = a.view(view).copy()
                want = O.ntt_gl64(x, inverse=bool(d)) if gl else O.ntt_u32(x, root, p, inverse=bool(d))
                assert np.array_equal(res, want), i
            # the same request alone
            out[:] = 0
            assert sv.submit(reqs[i]) == 0
            assert sv.wait_idle(30.0) == 0
            assert np.array_equal(out.view(view), res), i
        sv.poll()
        s = sv.stats()
        assert s["completed"] == 2 * len(reqs) and s["failed"] == 0
        assert s["peak_inflight"] >= 2  # requests overlapped on the device
    finally:
        sv.close()


def test_admission_waits_for_memory(ctx):
    # a 1 MiB arena: Goldilocks 2^16 polymul requests need 1 MiB each, so they run one at a time
    sv = st.Server(ctx, streams=4, max_log_n=16, arena_bytes=1 << 20)
    try:
        n = 1 << 16
        bufs, reqs = [], []
        for i in range(6):
            ta, a = _pinned(n, torch.int64)
            tb, b = _pinned(n, torch.int64)
            to, o = _pinned(n, torch.int64)
            a.view(np.uint64)[: n // 2] = O.uniform_u64(i, n // 2)
            b.view(np.uint64)[: n // 2] = O.uniform_u64(100 + i, n // 2)
            bufs.append((ta, tb, to, a, b, o))
            reqs.append(st.Request(st.REQ_POLYMUL, st.FIELD_GL64, 16, 0, 0, 0, i, ta.data_ptr(), tb.data_ptr(),
                                   to.data_ptr()))
        comps = sv.run_trace(reqs, [0.0] * len(reqs))
        assert all(c.status == 0 for c in comps)
        s = sv.stats()
        assert s["peak_arena_used"] <= s["arena_bytes"] == 1 << 20
        assert s["peak_inflight"] == 1
        x = bufs[0][3].view(np.uint64)[: n // 2].copy()
        y = bufs[0][4].view(np.uint64)[: n // 2].copy()
        ref = bufs[0][5].view(np.uint64)
        # spot-check the first product against the library's own polymul on device
        da = torch.from_numpy(bufs[0][3].copy()).cuda()
        db = torch.from_numpy(bufs[0][4].copy()).cuda()
        ctx.polymul_gl64(da, db, da, 16)
        torch.cuda.synchronize()
        assert np.array_equal(da.cpu().numpy().view(np.uint64), ref)
        # an operand larger than the arena is refused
        big = st.Request(st.REQ_POLYMUL, st.FIELD_GL64, 17, 0, 0, 0, 99, bufs[0][0].data_ptr(),
                         bufs[0][1].data_ptr(), bufs[0][2].data_ptr())
        assert sv.submit(big) == 5  # STNTT_EUNSUPPORTED (max_log_n 16)
        del x, y
    finally:
        sv.close()


def test_serving_full_size_range(ctx):
    """The serving configuration's size range, 2^12..2^22 in both fields with
    polynomial products: a seeded trace of 40 requests at 20k requests/s. Every
    transform is checked against the oracle, every product against the
    oracle's cyclic convolution (forward, element-wise product, inverse), and
    every result against the same request run alone."""
    sv = st.Server(ctx, streams=8, max_log_n=22)
    try:
        reqs, arr, keep, expect = _make_trace(7, 40, 12, 22, rate=20000.0)
        assert max(k[9] for k in keep) >= 20 and any(k[8] for k in keep)
        comps = sv.run_trace(reqs, arr)
        assert all(c.status == 0 for c in comps)
        mix = [k[5].copy() for k in keep]
        for i, (ta, tb, to, a, b, out, view, gl, poly, lg, d, p, root) in enumerate(keep):
            res = mix[i].view(view)
            x = a.view(view).copy()
            if poly:
                y = b.view(view).copy()
                want = O.cyclic_conv_gl64(x, y) if gl else O.cyclic_conv_u32(x, y, root, p)
                if expect[i] is not None:
                    assert np.array_equal(want[: expect[i].size], expect[i]), i
            else:
                want = O.ntt_gl64(x, inverse=bool(d)) if gl else O.ntt_u32(x, root, p, inverse=bool(d))
            assert np.array_equal(res, want), (i, lg, gl, poly)
            out[:] = 0
            assert sv.submit(reqs[i]) == 0
            assert sv.wait_idle(60.0) == 0
            assert np.array_equal(out.view(view), res), i
        assert sv.stats()["failed"] == 0
    finally:
        sv.close()
