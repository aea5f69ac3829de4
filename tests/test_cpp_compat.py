"""The C++ drop-in header (include/stntt_compat.hpp): it compiles against the
C ABI with the reference's call shapes, links with libstntt, and (on a GPU)
reproduces the reference's nttStockham results."""

import hashlib
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import stntt_gb300 as st

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "compat_check.cpp"


def _fnv(a: np.ndarray) -> str:
    return f"{O.fnv1a64(a.astype('<i4')):016x}"


def _build(tmp_path: Path) -> Path:
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "compat_check"
    so_dir = st.SO_PATH.parent
    cmd = ["g++", "-std=c++20", "-O1", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe), f"-L{so_dir}", "-lstntt",
           f"-Wl,-rpath,{so_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compat_header_compiles_and_links(stntt_lib, tmp_path):
    exe = _build(tmp_path)
    assert exe.exists()


@pytest.mark.gpu
def test_compat_header_matches_reference(stntt_lib, golden, tmp_path):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = _build(tmp_path)
    stream = O.ref_rng_vector(10 << 16)
    r = subprocess.run([str(exe)], input=" ".join(map(str, stream.tolist())), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-1].startswith("invalid_argument: size (12) must be a power of 2")
    by_case = {(c["log_n"], c["batch"]): c for c in golden["stockham"]}
    for ln in lines[:-1]:
        lg, b, h = ln.split()
        lg, b = int(lg), int(b)
        case = by_case[(lg, b)]
        # the reference's output for this case, restated by the oracle (pinned to the same digests)
        out = O.ntt_ref_wrap(stream[: (1 << lg) * b], case["root"], case["mod"], batch=b)
        assert hashlib.sha256(out.astype("<i4").tobytes()).hexdigest() == case["sha256"]
        assert h == _fnv(out), (lg, b)
