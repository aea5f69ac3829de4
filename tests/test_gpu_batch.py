"""Uneven batches in one persistent launch (stntt_ntt_batch / stntt_batch_*).

Every job is checked bit for bit against the CPU oracle and against one
launch sequence per job; a reusable batch is replayed from a CUDA graph; a
bounded device-side wait is made to run out and must report STNTT_ETIMEOUT.
"""

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _make_jobs(seed, n_jobs, lo, hi, fields=("gl64", "u32"), extra=()):
    rng = np.random.default_rng(seed)
    jobs, bufs, inputs, meta = [], [], [], []
    sizes = list(rng.integers(lo, hi + 1, n_jobs)) + list(extra)
    for i, lg in enumerate(sizes):
        lg = int(lg)
        inv = i % 2
        field = fields[i % len(fields)]
        if field == "u32":
            p, root = st.params_u32(lg)
            x = O.uniform_u32(seed * 10000 + i, p, 1 << lg)
            d = torch.from_numpy(x.view(np.int32).copy()).cuda()
            jobs.append(st.Job(st.FIELD_U32, lg, inv, p, root, 0, d.data_ptr()))
            meta.append(("u32", lg, inv, p, root))
        else:
            x = O.uniform_u64(seed * 10000 + i, 1 << lg)
            d = torch.from_numpy(x.view(np.int64).copy()).cuda()
            jobs.append(st.Job(st.FIELD_GL64, lg, inv, 0, 0, 0, d.data_ptr()))
            meta.append(("gl64", lg, inv, 0, 0))
        bufs.append(d)
        inputs.append(x)
    return jobs, bufs, inputs, meta


def _expected(x, m):
    field, lg, inv, p, root = m
    if field == "u32":
        return O.ntt_u32(x, root, p, inverse=bool(inv))
    return O.ntt_gl64(x, inverse=bool(inv))


def _host(d):
    a = d.cpu().numpy()
    return a.view(np.uint32) if d.dtype == torch.int32 else a.view(np.uint64)


def test_batch_matches_oracle_and_per_call(ctx):
    # mixed fields, directions and sizes, incl. tiny (< 2^4) and three-pass (2^25) jobs
    jobs, bufs, inputs, meta = _make_jobs(3, 120, 4, 18, extra=(0, 1, 2, 3, 25))
    ref_bufs = [b.clone() for b in bufs]
    ctx.ntt_batch(jobs)
    torch.cuda.synchronize()
    for b, x, m in zip(bufs, inputs, meta):
        assert np.array_equal(_host(b), _expected(x, m)), m
    # per-call path on the same inputs gives the same bits
    jobs2 = [st.Job(j.field, j.log_n, j.dir, j.p, j.root, 0, rb.data_ptr()) for j, rb in zip(jobs, ref_bufs)]
    ctx.ntt_batch(jobs2, per_call=True)
    torch.cuda.synchronize()
    for b, rb in zip(bufs, ref_bufs):
        assert torch.equal(b, rb)


def test_batch_reference_mix_shape(ctx):
    """The batched configuration's shape: Goldilocks, log2 n in [10, 18], half
    forward and half inverse (a smaller count of jobs)."""
    jobs, bufs, inputs, meta = _make_jobs(11, 256, 10, 18, fields=("gl64",))
    b = ctx.batch_create(jobs)
    info = b.info()
    assert info["fallback_jobs"] == 0 and info["items"] > 0
    b.launch()
    torch.cuda.synchronize()
    assert b.status() == 0
    for d, x, m in zip(bufs, inputs, meta):
        assert np.array_equal(_host(d), _expected(x, m)), m
    b.close()


def test_batch_graph_replay(ctx):
    jobs, bufs, inputs, meta = _make_jobs(21, 40, 6, 17)
    b = ctx.batch_create(jobs)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.launch(stream=s)
    # capture does not run the work; each replay transforms in place once
    for rep in range(2):
        for d, x in zip(bufs, inputs):
            d.copy_(torch.from_numpy(x.view(np.int32 if d.dtype == torch.int32 else np.int64).copy()))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert b.status() == 0
        for d, x, m in zip(bufs, inputs, meta):
            assert np.array_equal(_host(d), _expected(x, m)), (rep, m)
    b.close()


def test_bounded_wait_reports_timeout(ctx):
    assert ctx.selftest_wait_timeout(20000) == 4  # STNTT_ETIMEOUT
    # the context stays usable afterwards
    x = O.uniform_u64(5, 1 << 12)
    d = torch.from_numpy(x.view(np.int64).copy()).cuda()
    ctx.ntt_gl64(d, 12)
    torch.cuda.synchronize()
    assert np.array_equal(_host(d), O.ntt_gl64(x))


def test_batched_plan_splits(ctx):
    """stntt_set_plan_batched: jobs of the persistent launch take the split set
    for their size (one pass, or from 2^13 points two of 2^4..2^13 points,
    including uneven ones), bit-exact with the oracle."""
    splits = {12: [12], 13: [4, 9], 14: [9, 5], 16: [5, 11], 17: [7, 10], 18: [7, 11]}
    try:
        for lg, sp in splits.items():
            ctx.set_plan(st.FIELD_GL64, lg, sp, batched=True)
            ctx.set_plan(st.FIELD_U32, lg, sp, batched=True)
        jobs, bufs, inputs, meta = _make_jobs(11, 40, 12, 18)
        b = ctx.batch_create(jobs)
        assert b.info()["fallback_jobs"] == 0
        b.launch()
        torch.cuda.synchronize()
        assert b.status() == 0
        for d, x, m in zip(bufs, inputs, meta):
            assert np.array_equal(_host(d), _expected(x, m)), m
        b.close()
        with pytest.raises(st.StnttError):
            ctx.set_plan(st.FIELD_GL64, 20, [4, 8, 8], batched=True)  # three passes: not in the persistent launch
        with pytest.raises(st.StnttError):
            ctx.set_plan(st.FIELD_GL64, 14, [2, 12], batched=True)  # tiles below 2^4 points
        with pytest.raises(st.StnttError):
            ctx.set_plan(st.FIELD_GL64, 12, [6, 6], batched=True)  # two passes below 2^13 points
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)


def test_full_reference_mix_matches_per_call(ctx):
    """The batched configuration at full size: 4096 Goldilocks jobs, log2 n
    uniform in [10, 18] from the benchmark's seed, alternating forward /
    inverse (about 2.4e8 elements). The persistent launch, replayed from a
    CUDA graph, must equal one launch sequence per transform bit for bit on
    the same inputs; 48 jobs spread over the list are also checked against
    the oracle."""
    sizes = [int(v) for v in np.random.default_rng(0x57170001 + 3).integers(10, 19, 4096)]
    total = sum(1 << s for s in sizes)
    data = torch.empty(total, dtype=torch.int64, device="cuda")
    st.fill_uniform_gl64(data, 4242)
    torch.cuda.synchronize()
    ref = data.clone()
    jobs, jobs_ref, offs, off = [], [], [], 0
    for i, s in enumerate(sizes):
        jobs.append(st.Job(st.FIELD_GL64, s, i % 2, 0, 0, 0, data.data_ptr() + 8 * off))
        jobs_ref.append(st.Job(st.FIELD_GL64, s, i % 2, 0, 0, 0, ref.data_ptr() + 8 * off))
        offs.append(off)
        off += 1 << s
    sample = list(range(0, 4096, 4096 // 48))[:48]
    inputs = {i: data[offs[i]: offs[i] + (1 << sizes[i])].cpu().numpy().view(np.uint64).copy() for i in sample}
    b = ctx.batch_create(jobs)
    assert b.info()["fallback_jobs"] == 0
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.launch(stream=s)
    g.replay()
    torch.cuda.synchronize()
    assert b.status() == 0
    ctx.ntt_batch(jobs_ref, per_call=True)
    torch.cuda.synchronize()
    assert torch.equal(data, ref)
    for i in sample:
        got = data[offs[i]: offs[i] + (1 << sizes[i])].cpu().numpy().view(np.uint64)
        assert np.array_equal(got, O.ntt_gl64(inputs[i], inverse=bool(i % 2))), (i, sizes[i])
    b.close()
    del data, ref


@pytest.mark.parametrize("field", ["gl64", "u32"])
def test_batch_vector_lines_items_and_unaligned_fallback(ctx, field):
    """Two-pass jobs run their items in the vector-lines layout when every job
    of their class is 16-byte aligned; a class with a job off 16-byte
    alignment falls back to the 16-points-per-thread items. Both against the
    oracle, both directions, both fields."""
    sizes = [14, 14, 15, 15, 17, 18]
    offs = [0, 0, 0, 1, 0, 0]  # the 2^15 class gets one job off 16-byte alignment
    w = 8 if field == "gl64" else 4
    step = 16 // w
    total = sum((1 << s) + step for s in sizes)
    dt = torch.int64 if field == "gl64" else torch.int32
    buf = torch.zeros(total, dtype=dt, device="cuda")
    jobs, views, inputs, params = [], [], [], []
    pos = 0
    for i, (s, o) in enumerate(zip(sizes, offs)):
        if field == "gl64":
            x = O.uniform_u64(4242 + i, 1 << s)
            src = torch.from_numpy(x.view(np.int64))
            p = root = 0
        else:
            p, root = st.params_u32(s)
            x = O.uniform_u32(4242 + i, p, 1 << s)
            src = torch.from_numpy(x.view(np.int32))
        v = buf[pos + o: pos + o + (1 << s)]
        v.copy_(src)
        jobs.append(st.Job(st.FIELD_GL64 if field == "gl64" else st.FIELD_U32, s, i % 2, p, root, 0, v.data_ptr()))
        views.append(v)
        inputs.append(x)
        params.append((p, root))
        pos += (1 << s) + step
    assert views[3].data_ptr() % 16 != 0 and views[2].data_ptr() % 16 == 0
    ctx.ntt_batch(jobs)
    torch.cuda.synchronize()
    for i, (v, x, (p, root)) in enumerate(zip(views, inputs, params)):
        if field == "gl64":
            want = O.ntt_gl64(x, inverse=bool(i % 2))
            got = v.cpu().numpy().view(np.uint64)
        else:
            want = O.ntt_u32(x, root, p, inverse=bool(i % 2))
            got = v.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, want), (field, sizes[i])


def test_batch_u32_prime_above_2e29_keeps_plain_items(ctx):
    """A 32-bit batch with one job over a prime in [2^29, 2^30) runs its
    two-pass classes on the 16-points-per-thread items (the vector-lines
    items need 8p < 2^32); every job, the per-size primes' too, against the
    oracle."""
    sizes = [14, 15, 17, 15]
    jobs, bufs, inputs, params = [], [], [], []
    for i, s in enumerate(sizes):
        if i == 3:
            root, p = st.findParams(1 << s, 1 << 29)
            assert (1 << 29) <= p < (1 << 30)
        else:
            p, root = st.params_u32(s)
        x = O.uniform_u32(515 + i, p, 1 << s)
        d = torch.from_numpy(x.view(np.int32).copy()).cuda()
        jobs.append(st.Job(st.FIELD_U32, s, i % 2, p, root, 0, d.data_ptr()))
        bufs.append(d)
        inputs.append(x)
        params.append((p, root))
    ctx.ntt_batch(jobs)
    torch.cuda.synchronize()
    for i, (d, x, (p, root)) in enumerate(zip(bufs, inputs, params)):
        want = O.ntt_u32(x, root, p, inverse=bool(i % 2))
        assert np.array_equal(d.cpu().numpy().view(np.uint32), want), (i, sizes[i])


def test_batched_plan_with_vector_flag_keeps_checks(ctx):
    """A batched-launch plan whose passes carry STNTT_PASS_VEC does not put
    unaligned jobs on the vector-lines items: the batch's own alignment check
    decides. Against the oracle."""
    try:
        ctx.set_plan(st.FIELD_GL64, 15, [7, 8], elems=[8 | st.PASS_VEC] * 2, cols=[8, 8], batched=True)
        buf = torch.zeros(2 * (1 << 15) + 4, dtype=torch.int64, device="cuda")
        xs = [O.uniform_u64(77 + i, 1 << 15) for i in range(2)]
        views = [buf[1: 1 + (1 << 15)], buf[(1 << 15) + 3: (1 << 15) + 3 + (1 << 15)]]
        for v, x in zip(views, xs):
            v.copy_(torch.from_numpy(x.view(np.int64)))
        assert all(v.data_ptr() % 16 == 8 for v in views)
        jobs = [st.Job(st.FIELD_GL64, 15, i, 0, 0, 0, v.data_ptr()) for i, v in enumerate(views)]
        ctx.ntt_batch(jobs)
        torch.cuda.synchronize()
        for i, (v, x) in enumerate(zip(views, xs)):
            assert np.array_equal(v.cpu().numpy().view(np.uint64), O.ntt_gl64(x, inverse=bool(i)))
    finally:
        ctx.clear_plans()
        from stntt_gb300 import tune
        tune.apply_cache(ctx)
