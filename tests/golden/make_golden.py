"""Generate tests/golden/reference_vectors.json from the UNMODIFIED reference.

Run in a checkout where the reference sources exist (``make -C oracle ref``
compiles src/ntt/ntt_cpu.cpp and src/ntt/ntt_util.cpp in place, with
oracle/ref_shim.cpp, into oracle/_ref/libstntt_ref.so):

    python tests/golden/make_golden.py

Cases follow the reference's own doctest suite
(src/tests/cuda/ntt/st_ntt_test.cu:16-97): inputs are util::Rng(42) draws
(mt19937 + uniform_int<int>{0,9}, src/util/rng.h), the first size*batches
values of one stream; n = 2^2..2^20 with batches {1, 2, 5, 10}
(ntt_kernel.cuh:26), plus the suite's skipped range 2^21..2^26 at batch 1.
Outputs are stored as SHA-256 digests of the little-endian int32 bytes,
with the full vectors for small n. The nttCt / inttGs / pwc_convolution
cases pin the orderings and the convolution semantics of ntt_cpu.cpp:11-193.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_vectors.json"
BATCHES = [1, 2, 5, 10]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).astype("<i4").tobytes()).hexdigest()


def main() -> None:
    oracle.build(ref=True)
    R = oracle.ref()
    if R is None:
        raise SystemExit("oracle/_ref/libstntt_ref.so is missing (needs the reference checkout)")
    stream = np.empty((1 << 26), np.int32)
    R.ref_rng_vector(42, stream, stream.size)
    doc = {
        "source": "AlvaroPardoFente/stNTT src/ntt/ntt_cpu.cpp + ntt_util.cpp, compiled unmodified",
        "rng": {"seed": 42, "first64": stream[:64].tolist(), "sha256_2^26": sha(stream)},
        "params": {},
        "stockham": [],
        "nttct": [],
        "inttgs": [],
        "pwc": [],
    }
    for lg in range(0, 27):
        r, m = C.c_uint64(), C.c_uint64()
        assert R.ref_find_params(1 << lg, 11, C.byref(r), C.byref(m)) == 0
        doc["params"][str(lg)] = [r.value, m.value]  # (root, mod), findParams order
    for lg in range(2, 27):
        n = 1 << lg
        root, mod = doc["params"][str(lg)]
        for b in (BATCHES if lg <= 20 else [1]):
            x = stream[: n * b].copy()
            assert R.ref_ntt_stockham_batch(x, n, root, mod, b) == 0
            case = {"log_n": lg, "batch": b, "root": root, "mod": mod, "sha256": sha(x)}
            if n * b <= 256:
                case["out"] = x.tolist()
            doc["stockham"].append(case)
        print("stockham", lg, flush=True)
    for lg in range(1, 9):
        n = 1 << lg
        root, mod = doc["params"][str(lg)]
        x = stream[:n].copy()
        assert R.ref_ntt_ct(x, n, root, mod) == 0
        doc["nttct"].append({"log_n": lg, "root": root, "mod": mod, "in": stream[:n].tolist(), "out": x.tolist()})
        y = x.copy()
        assert R.ref_intt_gs(y, n, root, mod) == 0
        doc["inttgs"].append({"log_n": lg, "root": root, "mod": mod, "in": x.tolist(), "out": y.tolist()})
    for ln in (4, 8, 16, 64, 256):
        a = stream[1000:1000 + ln] + 1  # the reference requires positive entries
        b = stream[3000:3000 + ln] + 1
        out = np.empty(ln, np.int32)
        rr, mm = C.c_int32(), C.c_int32()
        assert R.ref_pwc_convolution(a.copy(), b.copy(), ln, out, C.byref(rr), C.byref(mm)) == 0
        doc["pwc"].append({"len": ln, "a": a.tolist(), "b": b.tolist(), "out": out.tolist(),
                           "root": rr.value, "mod": mm.value})
    OUT.write_text(json.dumps(doc, indent=0))
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
