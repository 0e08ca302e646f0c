"""Build the CPU oracle shared library (test infrastructure, never the product).

``python oracle/build.py`` compiles ``oracle/ss_oracle.c`` into
``oracle/_build/libss_oracle.so`` with OpenMP and without FMA contraction
(``-ffp-contract=off``), so the restated reference expressions round the way
a plain FP64 build of the reference does.
"""
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libss_oracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "ss_oracle.c"
    hdr = HERE / "ss_oracle.h"
    if (not force and OUT.exists() and OUT.stat().st_mtime > max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(f".{os.getpid()}.tmp.so")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-D_GNU_SOURCE", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
