"""CPU oracle for the stNTT hot path -- TEST INFRASTRUCTURE.

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package. It is the checker, never the product: the
CUDA library neither links nor calls it.

``lib()`` loads this project's C restatement of the reference CPU algorithms
(``stntt_oracle.c``; built by ``make`` in this folder). ``ref()`` loads the
unmodified reference CPU sources compiled by ``make ref`` (only where the
reference checkout exists); it is used to generate ``tests/golden``.
"""

from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
GL_P = 0xFFFFFFFF00000001

_lib = None
_ref = None

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def ref_sources() -> Path | None:
    """The reference sources the baselines compile from: $STNTT_REF_DIR, else
    the copy staged in baseline/_ref (``make -C oracle ref-stage REF=...``)."""
    for cand in (os.environ.get("STNTT_REF_DIR"), str(HERE.parent / "baseline" / "_ref")):
        if cand and (Path(cand) / "src" / "ntt" / "ntt_cpu.cpp").exists():
            return Path(cand)
    return None


def build(ref: bool = False) -> None:
    """Compile the oracle library (and, with ``ref``, the reference CPU code
    and the reference GPU benchmark driver)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if ref:
        src = ref_sources()
        env = dict(os.environ, REF=str(src)) if src else None
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True, env=env)
        # the reference's CUDA code (nvcc, sm_100): a missing toolkit only costs that baseline
        r = subprocess.run(["make", "-s", "-C", str(HERE), "ref-gpu"], env=env, capture_output=True, text=True)
        if r.returncode != 0:
            print(f"reference GPU benchmark not built: {r.stderr.strip()[-300:]}")


def ref_gpu_bench() -> Path | None:
    """The reference CUDA NTT benchmark driver built by ``make ref-gpu``."""
    exe = HERE / "_ref" / platform.machine() / "ref_gpu_bench"
    return exe if exe.exists() else None


def _bind(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


def lib():
    """The C restatement (built on first use)."""
    global _lib
    if _lib is None:
        so = HERE / "_lib" / platform.machine() / "libstntt_oracle.so"
        if not so.exists() or so.stat().st_mtime < (HERE / "stntt_oracle.c").stat().st_mtime:
            build()
        L = C.CDLL(str(so))
        u32, u64, i32, sz = C.c_uint32, C.c_uint64, C.c_int32, C.c_size_t
        _bind(L, "orc_mt19937_uniform_int", None, [u32, i32, i32, _i32p, sz])
        _bind(L, "orc_uniform_u32", None, [u64, u32, _u32p, sz])
        _bind(L, "orc_uniform_u64", None, [u64, u64, _u64p, sz])
        _bind(L, "orc_find_params", C.c_int, [u64, u64, C.POINTER(u64), C.POINTER(u64)])
        _bind(L, "orc_pow_mod", u64, [u64, u64, u64])
        _bind(L, "orc_gl_pow", u64, [u64, u64])
        _bind(L, "orc_gl_mul", u64, [u64, u64])
        _bind(L, "orc_gl_mul_slow", u64, [u64, u64])
        _bind(L, "orc_gl_root", u64, [u32])
        _bind(L, "orc_ntt_u32", C.c_int, [_u32p, u32, u32, u32, C.c_int])
        _bind(L, "orc_intt_u32", C.c_int, [_u32p, u32, u32, u32])
        _bind(L, "orc_ntt_gl64", C.c_int, [_u64p, u32, u64, C.c_int])
        _bind(L, "orc_intt_gl64", C.c_int, [_u64p, u32, u64])
        _bind(L, "orc_ntt_ref_wrap", C.c_int, [_i32p, i32, i32, i32, C.c_int])
        _bind(L, "orc_ntt_u32_batch", C.c_int, [_u32p, u32, u32, u32, u32, C.c_int, C.c_int])
        _bind(L, "orc_ntt_gl64_batch", C.c_int, [_u64p, u32, u32, C.c_int, C.c_int])
        _bind(L, "orc_ntt_ct_u32", C.c_int, [_u32p, u32, u32, u32])
        _bind(L, "orc_intt_gs_u32", C.c_int, [_u32p, u32, u32, u32])
        _bind(L, "orc_dft_u32", None, [_u32p, _u32p, u32, u32, u32])
        _bind(L, "orc_dft_gl64", None, [_u64p, _u64p, u32, u64])
        _bind(L, "orc_polymul_u32", None, [_u32p, sz, _u32p, sz, u32, _u32p])
        _bind(L, "orc_polymul_gl64", None, [_u64p, sz, _u64p, sz, _u64p])
        _bind(L, "orc_fnv1a64", u64, [C.c_void_p, sz])
        _bind(L, "orc_dft_point_u32", u32, [_u32p, u64, u32, u32, u64])
        _bind(L, "orc_dft_point_gl64", u64, [_u64p, u64, u64, u64])
        _bind(L, "orc_cyclic_conv_u32", C.c_int, [_u32p, _u32p, u32, u32, u32])
        _bind(L, "orc_cyclic_conv_gl64", C.c_int, [_u64p, _u64p, u32])
        _lib = L
    return _lib


def ref():
    """The unmodified reference CPU code, or None where it was not built."""
    global _ref
    if _ref is None:
        so = HERE / "_ref" / platform.machine() / "libstntt_ref.so"
        if not so.exists():
            return None
        try:
            R = C.CDLL(str(so))
        except OSError:  # e.g. built for another machine
            return None
        u64, i32 = C.c_uint64, C.c_int
        _bind(R, "ref_find_params", C.c_int, [u64, u64, C.POINTER(u64), C.POINTER(u64)])
        _bind(R, "ref_ntt_stockham", C.c_int, [_i32p, i32, i32, i32, i32])
        _bind(R, "ref_ntt_stockham_batch", C.c_int, [_i32p, i32, i32, i32, i32])
        _bind(R, "ref_ntt_ct", C.c_int, [_i32p, i32, i32, i32])
        _bind(R, "ref_intt_gs", C.c_int, [_i32p, i32, i32, i32])
        _bind(R, "ref_pwc_convolution", C.c_int, [_i32p, _i32p, i32, _i32p, C.POINTER(i32), C.POINTER(i32)])
        _bind(R, "ref_rng_vector", None, [i32, _i32p, C.c_size_t])
        _ref = R
    return _ref


# ---------------------------------------------------------------- wrappers
def find_params(size: int, min_mod: int = 11) -> tuple[int, int]:
    """findParams(size, min_mod) -> (root, mod) (src/ntt/ntt_util.cpp:10)."""
    r, m = C.c_uint64(), C.c_uint64()
    rc = lib().orc_find_params(size, min_mod, C.byref(r), C.byref(m))
    if rc:
        raise ValueError(f"find_params({size}, {min_mod}) failed: {rc}")
    return r.value, m.value


def ref_rng_vector(n: int, seed: int = 42) -> np.ndarray:
    """util::Rng(seed).get_vector(n): mt19937 + uniform_int<int>{0,9}."""
    out = np.empty(n, np.int32)
    lib().orc_mt19937_uniform_int(seed, 0, 9, out, n)
    return out


def uniform_u32(seed: int, p: int, n: int) -> np.ndarray:
    out = np.empty(n, np.uint32)
    lib().orc_uniform_u32(seed, p, out, n)
    return out


def uniform_u64(seed: int, n: int, p: int = GL_P) -> np.ndarray:
    out = np.empty(n, np.uint64)
    lib().orc_uniform_u64(seed, p, out, n)
    return out


def _log2(n: int) -> int:
    if n <= 0 or n & (n - 1):
        raise ValueError(f"size ({n}) must be a power of 2")
    return n.bit_length() - 1


def ntt_u32(vec, root: int, mod: int, inverse: bool = False, batch: int = 1, threads: int = 1) -> np.ndarray:
    """Field-exact Stockham NTT over Z/mod, natural order, batch contiguous."""
    v = np.ascontiguousarray(vec, dtype=np.uint32).copy()
    n = v.size // batch
    _log2(n)
    rc = lib().orc_ntt_u32_batch(v, n, batch, root, mod, int(inverse), threads)
    if rc:
        raise RuntimeError(f"orc_ntt_u32_batch rc={rc}")
    return v


def ntt_gl64(vec, inverse: bool = False, batch: int = 1, threads: int = 1) -> np.ndarray:
    v = np.ascontiguousarray(vec, dtype=np.uint64).copy()
    n = v.size // batch
    _log2(n)
    rc = lib().orc_ntt_gl64_batch(v, n, batch, int(inverse), threads)
    if rc:
        raise RuntimeError(f"orc_ntt_gl64_batch rc={rc}")
    return v


def ntt_ref_wrap(vec, root: int, mod: int, batch: int = 1, nsteps: int = -1) -> np.ndarray:
    """The reference's int32 wrap-around Stockham, restated in C."""
    v = np.ascontiguousarray(vec, dtype=np.int32).copy()
    n = v.size // batch
    for b in range(batch):
        seg = v[b * n:(b + 1) * n]
        buf = np.ascontiguousarray(seg)
        rc = lib().orc_ntt_ref_wrap(buf, n, root, mod, nsteps)
        if rc:
            raise RuntimeError(f"orc_ntt_ref_wrap rc={rc}")
        v[b * n:(b + 1) * n] = buf
    return v


def dft_u32(vec, root: int, mod: int) -> np.ndarray:
    x = np.ascontiguousarray(vec, dtype=np.uint32)
    out = np.empty_like(x)
    lib().orc_dft_u32(x, out, x.size, root, mod)
    return out


def dft_gl64(vec, root: int) -> np.ndarray:
    x = np.ascontiguousarray(vec, dtype=np.uint64)
    out = np.empty_like(x)
    lib().orc_dft_gl64(x, out, x.size, root)
    return out


def gl_root(log_n: int) -> int:
    return lib().orc_gl_root(log_n)


def polymul_u32(a, b, mod: int) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    out = np.empty(a.size + b.size - 1, np.uint32)
    lib().orc_polymul_u32(a, a.size, b, b.size, mod, out)
    return out


def polymul_gl64(a, b) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    out = np.empty(a.size + b.size - 1, np.uint64)
    lib().orc_polymul_gl64(a, a.size, b, b.size, out)
    return out


def cyclic_conv_u32(a, b, root: int, mod: int) -> np.ndarray:
    """Length-n cyclic convolution through the transform (pwcNtt semantics)."""
    x = np.ascontiguousarray(a, dtype=np.uint32).copy()
    y = np.ascontiguousarray(b, dtype=np.uint32).copy()
    if lib().orc_cyclic_conv_u32(x, y, x.size, root, mod):
        raise RuntimeError("orc_cyclic_conv_u32 failed")
    return x


def cyclic_conv_gl64(a, b) -> np.ndarray:
    x = np.ascontiguousarray(a, dtype=np.uint64).copy()
    y = np.ascontiguousarray(b, dtype=np.uint64).copy()
    if lib().orc_cyclic_conv_gl64(x, y, x.size):
        raise RuntimeError("orc_cyclic_conv_gl64 failed")
    return x


def ntt_ct_u32(vec, root: int, mod: int) -> np.ndarray:
    v = np.ascontiguousarray(vec, dtype=np.uint32).copy()
    if lib().orc_ntt_ct_u32(v, v.size, root, mod):
        raise RuntimeError("orc_ntt_ct_u32 failed")
    return v


def intt_gs_u32(vec, root: int, mod: int) -> np.ndarray:
    v = np.ascontiguousarray(vec, dtype=np.uint32).copy()
    if lib().orc_intt_gs_u32(v, v.size, root, mod):
        raise RuntimeError("orc_intt_gs_u32 failed")
    return v


def fnv1a64(a: np.ndarray) -> int:
    b = np.ascontiguousarray(a)
    return lib().orc_fnv1a64(b.ctypes.data, b.nbytes)


def cpu_count() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
