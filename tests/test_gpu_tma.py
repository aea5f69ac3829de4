"""TMA-staged passes (stntt_set_tma): bit-exact against the oracle and against
the plain kernels, over every tile geometry the staged kernel has -- column
passes (one or several 256-row boxes per tile), row passes with C <= n1,
n1 < C <= n1 n2 and whole small transforms (C > n1 n2, partial last tile),
both fields, forward and inverse -- plus the fallbacks (unaligned input,
fused pointwise product) and the bounded-wait self-test.
"""

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GL, U32 = st.FIELD_GL64, st.FIELD_U32


def dev64(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64).copy()).cuda()


def dev32(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32).copy()).cuda()


def host64(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint64)


def host32(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module")
def tctx(stntt_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = st.Context(0)
    c.set_tma(1)
    yield c
    torch.cuda.synchronize()
    c.close()


def run_gl(c, x, lg, batch, inverse=False):
    d = dev64(x)
    c.ntt_gl64(d, lg, batch, inverse=inverse)
    return host64(d)


def run_u32(c, x, lg, batch, p, root, inverse=False):
    d = dev32(x)
    c.ntt_u32(d, lg, batch, p, root, inverse=inverse)
    return host32(d)


# (log_n, batch, pass_logs or None for the context's plan, cols or None)
GL_CASES = [
    (7, 64, None, None),          # one pass, whole transforms of 128 points
    (8, 100, None, None),         # one pass, C > rows per transform, partial last tile
    (12, 5, None, None),          # one 4096-point row: 16 boxes of 256
    (16, 3, [8, 8], [16, 16]),    # column pass + row pass, C <= n1
    (19, 2, [5, 7, 7], [8, 16, 64]),  # row pass with n1 = 32 < C = 64 <= n1 n2
    (20, 1, [10, 10], None),      # 1024-point tiles (4 boxes per column tile)
    (22, 1, [11, 11], None),      # 2048-point tiles
    (24, 1, None, None),          # the tuned 2^24 plan (three 256-point passes)
]


@pytest.mark.parametrize("lg,batch,logs,cols", GL_CASES)
def test_gl64_staged_equals_oracle(tctx, lg, batch, logs, cols):
    if logs:
        tctx.clear_plans()  # without the packaged small-call shapes, calls under 2^22 elements take this plan too
        tctx.set_plan(GL, lg, logs, cols=cols)
    try:
        x = O.uniform_u64(700 + lg, batch << lg)
        f = run_gl(tctx, x, lg, batch)
        if batch << lg <= 1 << 22:
            assert np.array_equal(f, O.ntt_gl64(x, batch=batch, threads=8)), (lg, batch)
        back = run_gl(tctx, f, lg, batch, inverse=True)
        assert np.array_equal(back, x), (lg, batch)
        assert tctx.device_status() == 0
    finally:
        if logs:
            tctx.clear_plans()


U32_CASES = [
    (9, 40, None, None),
    (16, 4, [8, 8], [16, 16]),
    (18, 2, [9, 9], [4, 8]),       # 16-byte column boxes
    (21, 1, [7, 7, 7], None),
    (26, 1, None, None),           # the tuned 2^26 plan (three passes)
]


@pytest.mark.parametrize("lg,batch,logs,cols", U32_CASES)
def test_u32_staged_equals_plain(tctx, ctx, lg, batch, logs, cols):
    p, root = st.params_u32(lg)
    if logs:
        for c in (tctx, ctx):
            c.clear_plans()  # without the packaged small-call shapes, calls under 2^22 elements take this plan too
            c.set_plan(U32, lg, logs, cols=cols)
    try:
        x = O.uniform_u32(800 + lg, p, batch << lg)
        f = run_u32(tctx, x, lg, batch, p, root)
        assert np.array_equal(f, run_u32(ctx, x, lg, batch, p, root)), (lg, batch)
        if batch << lg <= 1 << 20:
            assert np.array_equal(f, O.ntt_u32(x, root, p, batch=batch)), (lg, batch)
        back = run_u32(tctx, f, lg, batch, p, root, inverse=True)
        assert np.array_equal(back, x), (lg, batch)
        assert tctx.device_status() == 0
    finally:
        if logs:
            tctx.clear_plans()
            ctx.clear_plans()


def test_staged_unaligned_input_falls_back(tctx):
    """An input 8 bytes past a 16-byte boundary cannot be a tensor-map base:
    the pass runs the plain kernel, with the same result."""
    lg, batch = 16, 2
    x = O.uniform_u64(901, (batch << lg) + 1)
    d = dev64(x)
    view = d[1:]
    assert view.data_ptr() % 16 == 8
    tctx.ntt_gl64(view, lg, batch)
    got = host64(d)
    assert got[0] == x[0]
    assert np.array_equal(got[1:], O.ntt_gl64(x[1:], batch=batch, threads=8))


def test_staged_polymul(tctx):
    """The polymul inverse fuses the pointwise product into its first pass
    (plain kernel); its row pass runs staged. Checked against schoolbook."""
    lg = 14
    n = 1 << lg
    h = n // 2
    a = np.zeros(n, np.uint64)
    b = np.zeros(n, np.uint64)
    a[:h] = O.uniform_u64(910, h)
    b[:h] = O.uniform_u64(911, h)
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    tctx.polymul_gl64(dev64(a), dev64(b), out, lg)
    want = O.polymul_gl64(a[:h], b[:h])
    assert np.array_equal(host64(out)[: want.size], want)
    assert tctx.device_status() == 0


def test_tma_wait_timeout_selftest(tctx):
    """A staged launch that issues no copy: its bounded wait runs out, the
    kernel reports STNTT_ETIMEOUT through the device word, and the context
    keeps working."""
    assert tctx.selftest_tma_timeout(2000) == 4
    assert tctx.device_status() == 0
    x = O.uniform_u64(920, 1 << 16)
    assert np.array_equal(run_gl(tctx, x, 16, 1), O.ntt_gl64(x))
