"""Build libslaterstoch.so (the CUDA library behind include/slaterstoch.h) for sm_103a.

Every translation unit in ``csrc/`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and linked into
``slater_stoch_gb300/_build/libslaterstoch.so``.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OUTDIR = HERE / "_build"
LIB = OUTDIR / "libslaterstoch.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    files = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((f.stat().st_mtime for f in files), default=0.0)


def _compile(src: Path, extra: list[str]) -> Path:
    obj = OUTDIR / (src.stem + ".o")
    if obj.exists() and obj.stat().st_mtime > max(src.stat().st_mtime, _deps_mtime()):
        return obj
    tmp = obj.with_suffix(f".{os.getpid()}.o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", str(INCLUDE), "-c", str(src), "-o", str(tmp), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, obj)
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OUTDIR.mkdir(parents=True, exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(os.cpu_count() or 8, len(srcs)))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.so")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
