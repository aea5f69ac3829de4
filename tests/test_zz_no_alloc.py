"""The allocation-free Goldilocks entry point (stntt_ntt_gl64_noalloc).

It serves callers that cannot call cudaMalloc: its scratch is a fixed array
inside the library instead of a context workspace. Called through the C ABI
and compared, bit for bit, with the regular entry point
(stntt_ntt_gl64_oop) and with the CPU oracle, forward and inverse, single
and batched, on two calls in a row. This file is named to be collected last.
"""

import ctypes as C

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64).copy()).cuda()


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint64)


def test_noalloc_matches_regular_entry_point(stntt_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fn = stntt_lib.stntt_ntt_gl64_noalloc
    ctx = st.Context(0)
    try:
        stream = torch.cuda.current_stream().cuda_stream
        cases = [(1, 1), (5, 3), (13, 1), (14, 2), (16, 1), (20, 1), (18, 4)]
        for call in range(2):  # two calls in a row reuse the shared scratch
            for lg, batch in cases:
                for inv in (0, 1):
                    x = O.uniform_u64(1000 * call + 10 * lg + inv, batch << lg)
                    src = _dev(x)
                    out_noalloc = torch.empty_like(src)
                    out_regular = torch.empty_like(src)
                    rc = fn(C.c_void_p(src.data_ptr()), C.c_void_p(out_noalloc.data_ptr()), lg, batch, inv,
                            C.c_void_p(stream))
                    assert rc == 0, (lg, batch, inv, rc)
                    ctx.ntt_gl64_oop(src, out_regular, lg, batch, inverse=bool(inv))
                    got = _host(out_noalloc)
                    assert np.array_equal(got, _host(out_regular)), (call, lg, batch, inv)
                    want = O.ntt_gl64(x, inverse=bool(inv), batch=batch)
                    assert np.array_equal(got, want), (call, lg, batch, inv)
                    assert np.array_equal(_host(src), x)  # input untouched
        # in place
        x = O.uniform_u64(7, 1 << 17)
        d = _dev(x)
        assert fn(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), 17, 1, 0, C.c_void_p(stream)) == 0
        assert np.array_equal(_host(d), O.ntt_gl64(x))
        # sizes beyond the fixed scratch are refused with STNTT_EUNSUPPORTED
        big = torch.empty(1 << 21, dtype=torch.int64, device="cuda")
        assert fn(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()), 21, 1, 0, C.c_void_p(stream)) == 5
        assert fn(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()), 20, 2, 0, C.c_void_p(stream)) == 5
        # a warm call does not take device memory (buffer sized for the 2^20 transform)
        d20 = _dev(O.uniform_u64(9, 1 << 20))
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        assert fn(C.c_void_p(d20.data_ptr()), C.c_void_p(d20.data_ptr()), 20, 1, 1, C.c_void_p(stream)) == 0
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0
    finally:
        ctx.close()
