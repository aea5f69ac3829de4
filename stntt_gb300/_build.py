"""In-tree build of libstntt.so (CUDA for sm_103a) -- no cmake, no pip.

``build()`` compiles each translation unit in parallel with nvcc and links
them into ``stntt_gb300/_lib/libstntt.so`` (the CUDA runtime linked
statically). Re-running only recompiles when a source is newer than its
object.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT = PKG / "_lib" / platform.machine()  # x86_64 here, aarch64 on the GPU hosts
SO = OUT / "libstntt.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "kernels_u32.cu", "kernels_u32l.cu", "kernels_gl64.cu", "kernels_gl64_f.cu", "kernels_gl64_i.cu",
           "kernels_tma_gl64.cu", "kernels_tma_u32l.cu", "kernels_v_gl64.cu", "kernels_v_gl64i.cu", "kernels_v_u32l.cu",
           "kernels_vc_gl64.cu", "kernels_vc_u32l.cu",
           "kernels_coop.cu", "noalloc.cu", "serve.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libstntt")
    return exe


def _flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-O2",
            f"-I{INCLUDE}", "-diag-suppress", "177"]


def _compile(src: str, extra: list[str]) -> Path:
    obj = OUT / (Path(src).stem + ".o")
    deps = [CSRC / src, *CSRC.glob("*.cuh"), *CSRC.glob("*.h"), *INCLUDE.glob("*.h")]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *_flags(), *extra, "-c", str(CSRC / src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    extra = list(extra or [])
    if verbose:
        extra += ["-Xptxas", "-v"]
    workers = min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if not SO.exists() or SO.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = SO.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared", *ARCH, "-cudart", "static", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, SO)
    return SO


if __name__ == "__main__":  # pragma: no cover
    print(build(verbose=True))
