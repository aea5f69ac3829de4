"""stntt_gb300 -- GB300-native number-theoretic transforms (Python host side).

This package is a thin ctypes layer over ``libstntt.so`` (the CUDA library in
``csrc/``, C ABI in ``include/stntt.h``). It mirrors the reference's host
interface for the hot path (AlvaroPardoFente/stNTT, ``src/ntt``):

* ``findParams(size, min_mod)`` -> ``(root, mod)``  (src/ntt/ntt_util.cpp:10)
* ``nttStockham(vec, size, root, mod, batches=1, nsteps=None)`` -- in place on a
  host int32 array, natural order in and out (src/ntt/ntt_cpu.cpp:46-90); the
  transform runs on the GPU. ``ref_wrap=True`` reproduces the reference's
  int32 wrap-around arithmetic bit for bit.
* ``Context`` -- device-buffer transforms on torch tensors, asynchronous on the
  current CUDA stream (replaces ``cuda::ntt::autoNtt<n>``,
  src/cuda/ntt/ntt_kernel.cuh:153-200).

There is no CPU fallback: every entry point raises ``StnttError`` when the
CUDA library is missing or fails.
"""

from __future__ import annotations

import ctypes as C
import os
import platform
from pathlib import Path
from typing import Iterable, Optional, Sequence

import numpy as np

__all__ = [
    "StnttError", "lib", "Context", "findParams", "params_u32", "gl64_root", "nttStockham",
    "GL_P", "FORWARD", "INVERSE", "FIELD_U32", "FIELD_GL64", "FLAG_REF_WRAP", "PASS_VEC", "Job",
]

PKG = Path(__file__).resolve().parent
SO_PATH = PKG / "_lib" / platform.machine() / "libstntt.so"
GL_P = 0xFFFFFFFF00000001
FORWARD, INVERSE = 0, 1
FIELD_U32, FIELD_GL64 = 0, 1
FLAG_REF_WRAP = 0x1
PASS_VEC = 0x100  # STNTT_PASS_VEC: elems flag for the vector-lines build of a pass
PASS_CLUSTER = 0x200  # STNTT_PASS_CLUSTER: with PASS_VEC | 8, the vector-lines cluster build (2^11..2^13 points)
STATUS = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ETIMEOUT", 5: "EUNSUPPORTED"}


class StnttError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"stntt {STATUS.get(status, status)}: {msg}")


class Job(C.Structure):
    """``stntt_job`` (include/stntt.h)."""

    _fields_ = [("field", C.c_uint32), ("log_n", C.c_uint32), ("dir", C.c_uint32), ("p", C.c_uint32),
                ("root", C.c_uint32), ("reserved", C.c_uint32), ("data", C.c_void_p)]


class Request(C.Structure):
    """``stntt_request`` (serving loop)."""

    _fields_ = [("kind", C.c_uint32), ("field", C.c_uint32), ("log_n", C.c_uint32), ("dir", C.c_uint32),
                ("p", C.c_uint32), ("root", C.c_uint32), ("id", C.c_uint64), ("in_a", C.c_void_p),
                ("in_b", C.c_void_p), ("out", C.c_void_p)]


class Completion(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("reserved", C.c_uint32), ("submit_s", C.c_double),
                ("start_s", C.c_double), ("done_s", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("streams", C.c_uint32), ("max_log_n", C.c_uint32), ("arena_bytes", C.c_uint64),
                ("prewarm_min_log_n", C.c_uint32), ("prewarm_max_log_n", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "admitted", "completed", "failed", "rejected",
                                          "peak_inflight", "arena_bytes", "peak_arena_used", "issue_ns", "poll_ns",
                                          "trace_late_max_ns", "trace_late_count")]


REQ_NTT, REQ_POLYMUL = 0, 1

_LIB = None
_vp, _u32, _u64, _i32, _sz, _int = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32, C.c_size_t, C.c_int

_SIGS = {
    "stntt_version": (_int, []),
    "stntt_status_string": (C.c_char_p, [_int]),
    "stntt_init": (_int, [C.POINTER(_vp), _int]),
    "stntt_destroy": (_int, [_vp]),
    "stntt_last_error": (C.c_char_p, [_vp]),
    "stntt_mem_usage": (_int, [_vp, C.POINTER(_sz)]),
    "stntt_release_stream": (_int, [_vp, _vp]),
    "stntt_last_kernel_ms": (_int, [_vp, C.POINTER(C.c_float)]),
    "stntt_find_params": (_int, [_u64, _u64, C.POINTER(_u64), C.POINTER(_u64)]),
    "stntt_find_params_device": (_int, [_u64, _u64, _vp, _vp]),
    "stntt_params_u32": (_int, [_u32, C.POINTER(_u32), C.POINTER(_u32)]),
    "stntt_gl64_root": (_int, [_u32, C.POINTER(_u64)]),
    "stntt_prepare": (_int, [_vp, _int, _u32, _u32, _u32, _int]),
    "stntt_plan_info": (_int, [_vp, _int, _u32, _u32, _u32, _int, C.POINTER(_u32), C.POINTER(_u32)]),
    "stntt_set_plan": (_int, [_vp, _int, _u32, _u32, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "stntt_set_plan_small": (_int, [_vp, _int, _u32, _u32, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "stntt_set_plan_batched": (_int, [_vp, _int, _u32, _u32, C.POINTER(_u32)]),
    "stntt_call_info": (_int, [_vp, _int, _u32, _u32, _u32, _u32, _int, C.POINTER(_u32), C.POINTER(_u32)]),
    "stntt_clear_plans": (_int, [_vp]),
    "stntt_device_key": (_int, [_int, C.c_char_p, _sz]),
    "stntt_ntt_u32": (_int, [_vp, _vp, _u32, _u32, _u32, _u32, _int, _u32, _vp]),
    "stntt_ntt_gl64": (_int, [_vp, _vp, _u32, _u32, _int, _vp]),
    "stntt_ntt_u32_oop": (_int, [_vp, _vp, _vp, _u32, _u32, _u32, _u32, _int, _vp]),
    "stntt_ntt_gl64_oop": (_int, [_vp, _vp, _vp, _u32, _u32, _int, _vp]),
    "stntt_ntt_u32_steps": (_int, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _u32, _vp]),
    "stntt_ntt_stockham_host": (_int, [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _u32]),
    "stntt_ntt_gl64_host": (_int, [_vp, _vp, _u32, _u32, _int]),
    "stntt_ntt_batch": (_int, [_vp, C.POINTER(Job), _sz, _vp]),
    "stntt_ntt_batch_per_call": (_int, [_vp, C.POINTER(Job), _sz, _vp]),
    "stntt_polymul_u32": (_int, [_vp, _vp, _vp, _vp, _u32, _u32, _u32, _vp]),
    "stntt_polymul_gl64": (_int, [_vp, _vp, _vp, _vp, _u32, _vp]),
    "stntt_pointwise_mul_u32": (_int, [_vp, _vp, _vp, _sz, _u32, _vp]),
    "stntt_pointwise_mul_gl64": (_int, [_vp, _vp, _vp, _sz, _vp]),
    "stntt_fill_uniform_u32": (_int, [_vp, _sz, _u64, _u32, _vp]),
    "stntt_fill_uniform_gl64": (_int, [_vp, _sz, _u64, _vp]),
    "stntt_ntt_gl64_noalloc": (_int, [_vp, _vp, _u32, _u32, _int, _vp]),
    "stntt_batch_create": (_int, [_vp, C.POINTER(Job), _sz, C.POINTER(_vp)]),
    "stntt_batch_launch": (_int, [_vp, _vp]),
    "stntt_batch_status": (_int, [_vp]),
    "stntt_batch_info": (_int, [_vp, C.POINTER(_sz), C.POINTER(_u32), C.POINTER(_sz)]),
    "stntt_batch_destroy": (_int, [_vp]),
    "stntt_selftest_wait_timeout": (_int, [_vp, _u32]),
    "stntt_set_tma": (_int, [_vp, _int]),
    "stntt_set_coop": (_int, [_vp, _int]),
    "stntt_device_status": (_int, [_vp]),
    "stntt_selftest_tma_timeout": (_int, [_vp, _u32]),
    "stntt_clock_s": (C.c_double, []),
    "stntt_measure_gl64_butterfly_rate": (_int, [_int, C.POINTER(C.c_double)]),
    "stntt_server_create": (_int, [_vp, C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "stntt_server_submit": (_int, [_vp, C.POINTER(Request)]),
    "stntt_server_submit_at": (_int, [_vp, C.POINTER(Request), C.c_double]),
    "stntt_server_poll": (_int, [_vp, C.POINTER(Completion), _sz, C.POINTER(_sz)]),
    "stntt_server_wait_idle": (_int, [_vp, C.c_double]),
    "stntt_server_stats_get": (_int, [_vp, C.POINTER(ServerStats)]),
    "stntt_server_run_trace": (_int, [_vp, C.POINTER(Request), C.POINTER(C.c_double), _sz, C.c_double,
                                      C.POINTER(Completion)]),
    "stntt_server_destroy": (_int, [_vp]),
}


def header_symbols() -> list[str]:
    """Every function name declared in include/stntt.h."""
    import re

    hdr = (PKG.parent / "include" / "stntt.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(stntt_\w+)\s*\(", hdr, re.M)))


def lib() -> C.CDLL:
    """Load libstntt.so; raises StnttError when it has not been built."""
    global _LIB
    if _LIB is None:
        if not SO_PATH.exists():
            raise StnttError(3, f"{SO_PATH} is missing: build it with __graft_entry__.build() "
                                "(there is no CPU fallback)")
        L = C.CDLL(str(SO_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _check(rc: int, ctx: Optional[int] = None) -> None:
    if rc != 0:
        msg = ""
        if ctx:
            raw = lib().stntt_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise StnttError(rc, msg)


# ---------------------------------------------------------------- parameters
def findParams(size: int, min_mod: int = 11) -> tuple[int, int]:
    """findParams(size, min_mod) -> (root, mod), src/ntt/ntt_util.cpp:10-14."""
    r, m = _u64(), _u64()
    _check(lib().stntt_find_params(size, min_mod, C.byref(r), C.byref(m)))
    return r.value, m.value


def find_params_device(size: int, min_mod: int, out, stream=None) -> None:
    """findParams on the device (stntt_find_params_device): writes
    (root, mod, status) into the int64 tensor `out` (3 elements) on `stream`."""
    _check(lib().stntt_find_params_device(size, min_mod, _ptr(out), _stream(stream)))


def params_u32(log_n: int) -> tuple[int, int]:
    """(p, root) = findParams(2^log_n, 11) as the reference's callers use it."""
    p, r = _u32(), _u32()
    _check(lib().stntt_params_u32(log_n, C.byref(p), C.byref(r)))
    return p.value, r.value


def gl64_root(log_n: int) -> int:
    r = _u64()
    _check(lib().stntt_gl64_root(log_n, C.byref(r)))
    return r.value


def gl64_butterfly_rate(device: int = 0) -> float:
    """Measured Goldilocks butterflies/s on register-resident data (integer roofline)."""
    r = C.c_double()
    _check(lib().stntt_measure_gl64_butterfly_rate(device, C.byref(r)))
    return r.value


def device_key(device: int = 0) -> str:
    buf = C.create_string_buffer(256)
    _check(lib().stntt_device_key(device, buf, 256))
    return buf.value.decode()


def _log2(n: int) -> int:
    if n <= 0 or n & (n - 1):
        raise StnttError(1, f"size ({n}) must be a power of 2")
    return n.bit_length() - 1


# ---------------------------------------------------------------- context
_DEFAULT: dict[int, "Context"] = {}


def _ptr(t) -> int:
    """Device pointer of a torch tensor (or a raw int)."""
    if isinstance(t, int):
        return t
    if not t.is_cuda:
        raise StnttError(1, "tensor must live on a CUDA device")
    if not t.is_contiguous():
        raise StnttError(1, "tensor must be contiguous")
    return t.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Context:
    """A ``stntt_ctx``: twiddle tables, plans and workspaces on one device."""

    def __init__(self, device: int = 0, tuned: bool = True):
        h = _vp()
        _check(lib().stntt_init(C.byref(h), device))
        self._h = h.value
        self.device = device
        if tuned and os.environ.get("STNTT_NO_TUNED_PLANS") != "1":
            from . import tune

            tune.apply_cache(self)  # the autotuner's plans for this GPU, if any

    @classmethod
    def default(cls, device: int = 0) -> "Context":
        if device not in _DEFAULT:
            _DEFAULT[device] = cls(device)
        return _DEFAULT[device]

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().stntt_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> int:
        return self._h

    def mem_usage(self) -> int:
        b = _sz()
        _check(lib().stntt_mem_usage(self._h, C.byref(b)), self._h)
        return b.value

    def release_stream(self, stream) -> None:
        """Free the scratch kept for `stream` (stntt_release_stream)."""
        _check(lib().stntt_release_stream(self._h, _stream(stream)), self._h)

    def last_kernel_ms(self) -> float:
        """Device time of the last host-buffer call (stntt_last_kernel_ms)."""
        ms = C.c_float()
        _check(lib().stntt_last_kernel_ms(self._h, C.byref(ms)), self._h)
        return ms.value

    def prepare(self, field: int, log_n: int, p: int = 0, root: int = 0, inverse: bool = False) -> None:
        _check(lib().stntt_prepare(self._h, field, log_n, p, root, INVERSE if inverse else FORWARD), self._h)

    def plan_info(self, field: int, log_n: int, p: int = 0, root: int = 0, inverse: bool = False):
        """(number of HBM passes, [log2 tile length per pass])."""
        n = _u32()
        logs = (_u32 * 4)()
        _check(lib().stntt_plan_info(self._h, field, log_n, p, root, INVERSE if inverse else FORWARD,
                                     C.byref(n), logs), self._h)
        return n.value, list(logs)[: n.value]

    def call_info(self, field: int, log_n: int, batch: int = 1, p: int = 0, root: int = 0, inverse: bool = False):
        """(kernel launches per call, [log2 tile length per pass]) for a call of this shape."""
        n = _u32()
        logs = (_u32 * 4)()
        _check(lib().stntt_call_info(self._h, field, log_n, batch, p, root, INVERSE if inverse else FORWARD,
                                     C.byref(n), logs), self._h)
        return n.value, [v for v in logs if v]

    def set_plan(self, field: int, log_n: int, pass_logs, elems=None, cols=None, small: bool = False,
                 batched: bool = False) -> None:
        """Override the plan shape for one size (stntt_set_plan); small=True sets
        the shape for calls of fewer than 2^22 elements (stntt_set_plan_small),
        batched=True the pass split of jobs in the persistent batched launch
        (stntt_set_plan_batched; elems and cols do not apply there)."""
        k = len(pass_logs)
        arr = lambda v: (_u32 * k)(*(v if v is not None else [0] * k))  # noqa: E731
        if batched:
            _check(lib().stntt_set_plan_batched(self._h, field, log_n, k, arr(pass_logs)), self._h)
            return
        fn = lib().stntt_set_plan_small if small else lib().stntt_set_plan
        _check(fn(self._h, field, log_n, k, arr(pass_logs), arr(elems), arr(cols)), self._h)

    def clear_plans(self) -> None:
        _check(lib().stntt_clear_plans(self._h), self._h)

    def set_tma(self, mode: int) -> None:
        """TMA-staged passes: -1 built-in choice, 0 never, 1 wherever a pass
        allows it (stntt_set_tma; drops cached plans)."""
        _check(lib().stntt_set_tma(self._h, mode), self._h)

    def set_coop(self, mode: int) -> None:
        """Small two-pass calls of 2^18..2^21 points as one cooperative launch:
        1 where the shape fits (default), 0 never (stntt_set_coop)."""
        _check(lib().stntt_set_coop(self._h, mode), self._h)

    def device_status(self) -> int:
        """STNTT_ETIMEOUT (4) when a staged pass gave up waiting for a copy
        since the last call, else 0 (stntt_device_status; synchronise first)."""
        return lib().stntt_device_status(self._h)

    def selftest_tma_timeout(self, spin_limit: int) -> int:
        """Status of a staged launch that issues no copy (expected: 4)."""
        return lib().stntt_selftest_tma_timeout(self._h, spin_limit)

    # -- device transforms (torch tensors: int32 storage for u32, int64 for gl64)
    def ntt_u32(self, data, log_n: int, batch: int, p: int, root: int, inverse: bool = False,
                ref_wrap: bool = False, stream=None) -> None:
        flags = FLAG_REF_WRAP if ref_wrap else 0
        _check(lib().stntt_ntt_u32(self._h, _ptr(data), log_n, batch, p, root, INVERSE if inverse else FORWARD,
                                   flags, _stream(stream)), self._h)

    def ntt_u32_oop(self, src, dst, log_n: int, batch: int, p: int, root: int, inverse: bool = False,
                    stream=None) -> None:
        _check(lib().stntt_ntt_u32_oop(self._h, _ptr(src), _ptr(dst), log_n, batch, p, root,
                                       INVERSE if inverse else FORWARD, _stream(stream)), self._h)

    def ntt_u32_steps(self, data, log_n: int, batch: int, p: int, root: int, nsteps: int,
                      ref_wrap: bool = False, stream=None) -> None:
        _check(lib().stntt_ntt_u32_steps(self._h, _ptr(data), log_n, batch, p, root, nsteps,
                                         FLAG_REF_WRAP if ref_wrap else 0, _stream(stream)), self._h)

    def ntt_gl64(self, data, log_n: int, batch: int = 1, inverse: bool = False, stream=None) -> None:
        _check(lib().stntt_ntt_gl64(self._h, _ptr(data), log_n, batch, INVERSE if inverse else FORWARD,
                                    _stream(stream)), self._h)

    def ntt_gl64_oop(self, src, dst, log_n: int, batch: int = 1, inverse: bool = False, stream=None) -> None:
        _check(lib().stntt_ntt_gl64_oop(self._h, _ptr(src), _ptr(dst), log_n, batch,
                                        INVERSE if inverse else FORWARD, _stream(stream)), self._h)

    def polymul_u32(self, a, b, out, log_n: int, p: int, root: int, stream=None) -> None:
        _check(lib().stntt_polymul_u32(self._h, _ptr(a), _ptr(b), _ptr(out), log_n, p, root, _stream(stream)),
               self._h)

    def polymul_gl64(self, a, b, out, log_n: int, stream=None) -> None:
        _check(lib().stntt_polymul_gl64(self._h, _ptr(a), _ptr(b), _ptr(out), log_n, _stream(stream)), self._h)

    def ntt_batch(self, jobs: Sequence[Job], per_call: bool = False, stream=None) -> None:
        arr = (Job * len(jobs))(*jobs)
        f = lib().stntt_ntt_batch_per_call if per_call else lib().stntt_ntt_batch
        _check(f(self._h, arr, len(jobs), _stream(stream)), self._h)

    # -- reusable batches (CUDA-graph friendly)
    def batch_create(self, jobs: Sequence[Job]) -> "Batch":
        arr = (Job * len(jobs))(*jobs)
        h = _vp()
        _check(lib().stntt_batch_create(self._h, arr, len(jobs), C.byref(h)), self._h)
        return Batch(self, h.value)

    def selftest_wait_timeout(self, spin_limit: int) -> int:
        """Status of a persistent launch whose only work item waits on a
        counter nothing sets (expected: 4, STNTT_ETIMEOUT)."""
        return lib().stntt_selftest_wait_timeout(self._h, spin_limit)

    # -- host arrays (synchronous)
    def ntt_stockham_host(self, vec: np.ndarray, size: int, root: int, mod: int, batches: int = 1,
                          nsteps: Optional[int] = None, ref_wrap: bool = False) -> np.ndarray:
        if vec.dtype != np.int32 or not vec.flags.c_contiguous:
            raise StnttError(1, "vec must be a C-contiguous int32 array")
        if vec.size < size * batches:
            raise StnttError(1, "vec is shorter than size * batches")
        _check(lib().stntt_ntt_stockham_host(self._h, vec.ctypes.data, size, root, mod, batches,
                                             -1 if nsteps is None else nsteps,
                                             FLAG_REF_WRAP if ref_wrap else 0), self._h)
        return vec

    def ntt_gl64_host(self, vec: np.ndarray, log_n: int, batch: int = 1, inverse: bool = False) -> np.ndarray:
        if vec.dtype != np.uint64 or not vec.flags.c_contiguous:
            raise StnttError(1, "vec must be a C-contiguous uint64 array")
        _check(lib().stntt_ntt_gl64_host(self._h, vec.ctypes.data, log_n, batch, INVERSE if inverse else FORWARD),
               self._h)
        return vec


class Batch:
    """A ``stntt_batch``: the work list of one uneven batch, launchable many
    times (``launch`` is capturable in a CUDA graph)."""

    def __init__(self, ctx: Context, handle: int):
        self.ctx, self._h = ctx, handle

    def launch(self, stream=None) -> None:
        _check(lib().stntt_batch_launch(self._h, _stream(stream)), self.ctx.handle)

    def status(self) -> int:
        return lib().stntt_batch_status(self._h)

    def info(self) -> dict:
        it, fb, gr = _sz(), _sz(), _u32()
        _check(lib().stntt_batch_info(self._h, C.byref(it), C.byref(gr), C.byref(fb)))
        return {"items": it.value, "grid": gr.value, "fallback_jobs": fb.value}

    def close(self) -> None:
        if self._h:
            lib().stntt_batch_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A ``stntt_server``: the request loop (see include/stntt.h)."""

    def __init__(self, ctx: Context, streams: int = 32, max_log_n: int = 22, arena_bytes: int = 0,
                 prewarm: tuple[int, int] | None = None):
        cfg = ServerConfig(streams, max_log_n, arena_bytes, *(prewarm or (0, 0)))
        h = _vp()
        _check(lib().stntt_server_create(ctx.handle, C.byref(cfg), C.byref(h)), ctx.handle)
        self.ctx, self._h = ctx, h.value

    def submit(self, req: Request) -> int:
        return lib().stntt_server_submit(self._h, C.byref(req))

    def wait_idle(self, timeout_s: float = 60.0) -> int:
        return lib().stntt_server_wait_idle(self._h, timeout_s)

    def poll(self, max_items: int = 4096) -> list:
        buf = (Completion * max_items)()
        got = _sz()
        _check(lib().stntt_server_poll(self._h, buf, max_items, C.byref(got)))
        return [buf[i] for i in range(got.value)]

    def run_trace(self, reqs: Sequence[Request], arrivals_s: Sequence[float], timeout_s: float = 120.0):
        n = len(reqs)
        r = (Request * n)(*reqs)
        a = (C.c_double * n)(*arrivals_s)
        out = (Completion * n)()
        rc = lib().stntt_server_run_trace(self._h, r, a, n, timeout_s, out)
        if rc not in (0,):
            raise StnttError(rc, "run_trace")
        return out

    def stats(self) -> dict:
        s = ServerStats()
        _check(lib().stntt_server_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self._h:
            lib().stntt_server_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def nttStockham(vec: np.ndarray, size: int, root: int, mod: int, batches: int = 1,
                nsteps: Optional[int] = None, ref_wrap: bool = False, device: int = 0) -> np.ndarray:
    """In-place forward NTT of a host int32 array on the GPU.

    Mirrors ``nttStockham(int *vec, int size, int root, int mod, nsteps)`` and
    ``nttStockham(std::span<int>, size, root, mod, batches, nsteps)``
    (src/ntt/ntt_cpu.h:8-9). Raises ``StnttError`` (EINVAL, "size (N) must be a
    power of 2") where the reference throws ``std::invalid_argument``.
    """
    return Context.default(device).ntt_stockham_host(vec, size, root, mod, batches, nsteps, ref_wrap)


# ---------------------------------------------------------------- inputs
def fill_uniform_u32(t, seed: int, p: int, stream=None) -> None:
    """Device-side uniform residues in [0, p) (counter-based splitmix64)."""
    _check(lib().stntt_fill_uniform_u32(_ptr(t), t.numel(), seed, p, _stream(stream)))


def fill_uniform_gl64(t, seed: int, stream=None) -> None:
    _check(lib().stntt_fill_uniform_gl64(_ptr(t), t.numel(), seed, _stream(stream)))


def uniform_u32_host(seed: int, p: int, n: int) -> np.ndarray:
    """Host copy of the same generator (numpy), for end-to-end host inputs."""
    return _uniform_host(seed, n, p, bits32=True).astype(np.uint32)


def uniform_gl64_host(seed: int, n: int) -> np.ndarray:
    return _uniform_host(seed, n, GL_P, bits32=False)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _uniform_host(seed: int, n: int, p: int, bits32: bool) -> np.ndarray:
    with np.errstate(over="ignore"):
        out = np.empty(n, np.uint64)
        todo = np.arange(n, dtype=np.uint64)
        attempt = 0
        limit = (1 << 32) - ((1 << 32) % p) if bits32 else p
        while todo.size:
            ctr = todo + np.uint64(attempt << 40) + np.uint64(1)
            z = _mix(np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) * ctr)
            if bits32:
                z = z >> np.uint64(32)
            ok = z < np.uint64(limit)
            vals = z[ok] % np.uint64(p) if bits32 else z[ok]
            out[todo[ok]] = vals
            todo = todo[~ok]
            attempt += 1
        return out
