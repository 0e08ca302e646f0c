"""ctypes loader for libslaterstoch.so (the C ABI declared in include/slaterstoch.h).

There is no CPU fallback: if the CUDA library is missing or cannot be loaded, every
call raises ``ExtensionMissing``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libslaterstoch.so"

i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
u16p = np.ctypeslib.ndpointer(np.uint16, flags="C")

# name -> (restype, argtypes); mirrors include/slaterstoch.h
SIGNATURES = {
    "ss_create": (C.c_void_p, [C.c_int, C.c_size_t]),
    "ss_destroy": (None, [C.c_void_p]),
    "ss_strerror": (C.c_char_p, [C.c_int]),
    "ss_last_error": (C.c_char_p, []),
    "ss_launch_count": (C.c_int64, [C.c_void_p]),
    "ss_basis_set": (C.c_int, [C.c_void_p, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, C.c_int,
                               f64p, f64p]),
    "ss_quartets_set": (C.c_int, [C.c_void_p, C.c_int64, i32p, i32p, i32p, i32p]),
    "ss_basis_systems": (C.c_int, [C.c_void_p, C.c_int, i32p]),
    "ss_precond": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ss_gauss_eri": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_zvmc": (C.c_int, [C.c_void_p, C.c_double, C.c_uint64, C.c_int64, C.c_int, C.c_int, C.c_int,
                          C.c_double, C.c_void_p, C.c_void_p]),
    "ss_zvmc_walkers": (C.c_int, [C.c_void_p, C.c_double, f64p, f64p, C.c_int64, C.c_int, C.c_int,
                                  C.c_void_p, C.c_void_p]),
    "ss_draw_walkers": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p]),
    "ss_shared_samples": (C.c_int, [C.c_void_p, C.c_double, C.c_uint64, C.c_int64, C.c_int64,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_combine": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ss_two_e_job": (C.c_int, [C.c_void_p, C.c_double, C.c_uint64, C.c_int64, C.c_int, C.c_int, C.c_int,
                               C.c_double, C.c_void_p, C.c_void_p]),
    "ss_job_submit": (C.c_int, [C.c_void_p, C.c_double, C.c_uint64, C.c_int64, C.c_int, C.c_int, C.c_int,
                                C.c_double, C.c_void_p]),
    "ss_job_submit_inputs": (C.c_int, [C.c_void_p, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, C.c_int, f64p,
                                       f64p, C.c_int64, i32p, i32p, i32p, i32p, C.c_double, C.c_uint64,
                                       C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p]),
    "ss_job_poll": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "ss_job_info": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_job_result": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "ss_write_one_e_matrix": (C.c_int, [C.c_char_p, C.c_int, f64p]),
    "ss_job_limits": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int]),
    "ss_job_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_job_footprint": (C.c_size_t, [C.c_int64]),
    "ss_nuclei_set": (C.c_int, [C.c_void_p, C.c_int, f64p, f64p]),
    "ss_one_e": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_write_bielec_ao": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ss_write_bielec_ao_arrays": (C.c_int, [C.c_char_p, C.c_int64, i32p, i32p, i32p, i32p, f64p, C.c_void_p]),
    "ss_invalidate": (C.c_int, [C.c_void_p]),
    "ss_mc_max_sigma": (C.c_double, [C.c_void_p]),
    "ss_mc_blocks_done": (C.c_int, [C.c_void_p]),
    "ss_stream": (C.c_void_p, [C.c_void_p]),
    "ss_split_bf16_gemm": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, u16p, u16p, u16p, u16p, C.c_int,
                                     f32p]),
    "ss_split_bf16_gemm_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "ss_psd_clean": (C.c_int, [C.c_void_p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64,
                               C.c_void_p]),
    "ss_davidson": (C.c_int, [C.c_void_p, f64p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p,
                              C.c_void_p]),
    "ss_psd_project": (C.c_int, [C.c_void_p, f64p, C.c_int, C.c_void_p]),
    "ss_monocenter": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ss_set_exact_monocenter": (C.c_int, [C.c_void_p, C.c_int]),
    "ss_set_eri_tiers": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    "ss_davidson_clean": (C.c_int, [C.c_void_p, f64p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                    C.c_void_p]),
}


class ExtensionMissing(RuntimeError):
    pass


class SSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"slaterstoch error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None):
    """Load the library (building it first only if explicitly asked via SS_BUILD=1)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists() and os.environ.get("SS_BUILD") == "1":
        from .build import build
        build()
    if not p.exists():
        raise ExtensionMissing(f"{p} not found: run `python -c 'import __graft_entry__ as g; g.build()'`")
    try:
        L = C.CDLL(str(p))
    except OSError as e:
        raise ExtensionMissing(f"cannot load {p}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int):
    if rc != 0:
        L = load()
        raise SSError(rc, (L.ss_last_error() or b"").decode() or L.ss_strerror(rc).decode())
