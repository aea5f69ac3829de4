"""The compile-time bound plans of the 32-bit vector-lines DFTs (lz_plan in
stntt_gb300/csrc/tile_v.cuh): a host program built from the same header
replays every planned network with worst-case inputs and checks that no value
reaches 8p (so the kernels' 32-bit arithmetic never wraps for p < 2^29), that
the outputs respect the plan's bound and stay congruent to the exact DIF
network, for every findParams prime up to n = 2^26 and the largest prime below
2^29. The GPU parity tests check the kernels themselves."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "lazy_bounds_check.cu"


def test_lazy_bound_plans(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path / "lazy_bounds_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-diag-suppress",
                        "177", f"-I{ROOT / 'stntt_gb300' / 'csrc'}", str(SRC), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "violations 0" in r.stdout
