"""Host build of the ERI kernel's arithmetic (tests/eri_host_shim.cpp over csrc/eri_kernel.cuh),
shared by the CPU tests of the kernel templates and the GPU parity tests that need the kernel's
own primitive-pair Schwarz factors (to pick the quartets where screening and the FP32 tier do
the most work).  Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "slater_stoch_gb300" / "csrc"
f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C")


def available() -> bool:
    return shutil.which("g++") is not None and shutil.which("nvcc") is not None


def build(outdir: Path, sanitize: bool = False) -> Path:
    """g++ build of the shim (the CUDA headers only provide the __host__/__device__ macros)."""
    cuda_inc = Path(shutil.which("nvcc")).resolve().parent.parent / "include"
    out = Path(outdir) / ("liberi_host_san.so" if sanitize else "liberi_host.so")
    flags = ["-O1", "-g", "-fsanitize=address,undefined,bounds", "-fno-omit-frame-pointer"] if sanitize else ["-O2"]
    subprocess.run(["g++", *flags, "-std=c++17", "-ffp-contract=off", "-Wno-unknown-pragmas", "-shared", "-fPIC",
                    f"-I{cuda_inc}", f"-I{CSRC}", str(HERE / "eri_host_shim.cpp"), "-o", str(out)], check=True)
    return out


def load(path: Path):
    L = C.CDLL(str(path))
    L.ss_host_eri.argtypes = [C.c_int, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, f64p, f64p, C.c_int64,
                              i32p, i32p, i32p, i32p, C.c_int, C.c_int, f64p, i32p]
    L.ss_host_eri.restype = C.c_int
    L.ss_host_fp32_error.argtypes = [C.c_int, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, f64p, f64p, C.c_int64,
                                     i32p, i32p, i32p, i32p, f64p, C.c_double, f64p]
    L.ss_host_fp32_error.restype = C.c_int
    L.ss_host_tier_counts.argtypes = [C.c_int, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, f64p, f64p, C.c_int64,
                                      i32p, i32p, i32p, i32p, f64p, C.c_double, C.c_double, f64p, i32p]
    L.ss_host_tier_counts.restype = C.c_int
    return L


def basis_arrays(b):
    return [np.ascontiguousarray(b.center, np.float64).reshape(-1), np.ascontiguousarray(b.npower, np.int32).reshape(-1),
            np.ascontiguousarray(b.n_sto, np.int32), np.ascontiguousarray(b.i_type, np.int32),
            np.ascontiguousarray(b.n_gauss, np.int32), np.ascontiguousarray(b.c_gauss, np.float64).reshape(-1),
            np.ascontiguousarray(b.g_gauss, np.float64).reshape(-1), np.ascontiguousarray(b.g_slater, np.float64)]


def tier_counts(L, b, quartets, pre, eps_screen=1e-18, eps32=1e-13):
    """Per quartet: (counts[nq, 4] = screened, FP32 tier, FP64, all primitive quartets;
    cls[nq, 3] = the kernel instance L, LK, tc), as the device splits them."""
    qq = [np.ascontiguousarray(x, np.int32) for x in quartets]
    nq = len(qq[0])
    counts = np.zeros(4 * nq)
    cls = np.zeros(3 * nq, np.int32)
    rc = L.ss_host_tier_counts(int(b.n), int(b.ld), *basis_arrays(b), nq, *qq,
                               np.ascontiguousarray(pre, np.float64).reshape(-1), float(eps_screen), float(eps32),
                               counts, cls)
    assert rc == 0
    return counts.reshape(nq, 4), cls.reshape(nq, 3)
