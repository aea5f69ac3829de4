"""The C-ABI library: builds, loads, exports what include/stntt.h declares.

No compute calls here (no GPU needed).
"""

import ctypes as C
import subprocess

import pytest

import stntt_gb300 as st


def test_exports_every_header_symbol(stntt_lib):
    names = st.header_symbols()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", str(st.SO_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(stntt_lib, n)


def test_find_params_matches_reference(stntt_lib, golden):
    for lg, (root, mod) in golden["params"].items():
        assert st.findParams(1 << int(lg), 11) == (root, mod), lg
    assert st.findParams(1000, 100000) == st.findParams(1000, 100000)


def test_params_u32_and_gl_root(stntt_lib, golden):
    for lg in range(0, 27):
        root, mod = golden["params"][str(lg)]
        assert st.params_u32(lg) == (mod, root)
    import oracle as O
    for lg in (0, 1, 10, 24, 32):
        assert st.gl64_root(lg) == O.gl_root(lg)
    with pytest.raises(st.StnttError):
        st.gl64_root(33)


def test_status_strings(stntt_lib):
    assert stntt_lib.stntt_status_string(0) == b"ok"
    assert stntt_lib.stntt_version() == 1


def test_no_cpu_fallback_without_gpu(stntt_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert stntt_lib.stntt_init(C.byref(h), 0) != 0
    with pytest.raises(st.StnttError):
        st.Context(0)


def test_header_compiles_as_c_and_links(stntt_lib, tmp_path):
    """include/stntt.h is plain C: a C11 host (tests/cpp/c_abi_check.c, the
    calls of a single transform, an uneven batch, device-side parameters, the
    TMA switch and the allocation-free entry point) compiles warning-free with
    -pedantic and links against libstntt."""
    import shutil
    from pathlib import Path

    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    root = Path(__file__).resolve().parents[1]
    exe = tmp_path / "c_abi_check"
    so_dir = st.SO_PATH.parent
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{root / 'include'}",
                        str(root / "tests" / "cpp" / "c_abi_check.c"), "-o", str(exe), f"-L{so_dir}", "-lstntt",
                        f"-Wl,-rpath,{so_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()
