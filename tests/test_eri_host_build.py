"""The analytic ERI kernel's arithmetic (csrc/eri_kernel.cuh) built for the host and checked
against the oracle on the CPU: the same templates, Boys tables, template-instance choice,
light-ket orientation ((jl|ik) with the lighter pair as the ket) and folded primitive pairs as
the device, without the device's screening and FP32 tier.

Gate (the GPU parity gate): |host - oracle| <= 1e-12 |oracle| + 1e-12 sqrt((ik|ik)(jl|jl)).
The light-ket instances, the full-L instances and the full-L instances with every quartet
evaluated as (jl|ik) agree with each other within the same gate."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import eri_host
from slater_stoch_gb300 import basis, configs, perfmodel

HERE = Path(__file__).resolve().parent
PRIM_FP32_EPS = 1e-11  # the kernel's default threshold of the FP32 tier (csrc/ss_common.cuh)
CSRC = HERE.parent / "slater_stoch_gb300" / "csrc"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not eri_host.available():
        pytest.skip("g++ or the CUDA headers not available")
    return eri_host.load(eri_host.build(tmp_path_factory.mktemp("eri")))


def _host_eri(lib, b, q, mode=0, fold=1):
    qq = [np.ascontiguousarray(x, np.int32) for x in q]
    out = np.zeros(len(qq[0]))
    lk = np.zeros(len(qq[0]), np.int32)
    rc = lib.ss_host_eri(int(b.n), int(b.ld), *eri_host.basis_arrays(b), len(qq[0]), *qq, mode, fold, out, lk)
    assert rc == 0
    return out, lk


def _gate(x, ref, pre, q, n):
    P = pre.reshape(n, n, order="F")
    i, j, k, l = [np.asarray(a) - 1 for a in q]
    bound = 1e-12 * np.abs(ref) + 1e-12 * np.sqrt(np.abs(P[i, k] * P[j, l]))
    return np.abs(x - ref) <= bound


@pytest.fixture(scope="module")
def h2o26(lib):
    from oracle import binding as O
    O.set_sum_mode("extended")
    b = configs.h2o_26(ng0=3)
    q = basis.build_mapping(b.n)
    ob = O.OracleBasis(b)
    pre = O.precond(ob)
    ref, _ = O.gauss_eri(ob, q)
    return b, q, pre, ref


def test_host_kernel_matches_oracle_h2o26(lib, h2o26):
    b, q, pre, ref = h2o26
    got, lk = _host_eri(lib, b, q, mode=0)
    cls = perfmodel.kernel_classes(b, q)
    assert (cls[:, 1] == lk).all()  # the Python classifier picks the instances the host build uses
    for L, LK in ((1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (3, 2), (4, 1), (4, 2)):  # every light-ket bound is exercised
        assert ((cls[:, 0] == L) & (lk == LK)).sum() > 0, (L, LK)
    ok = _gate(got, ref, pre, q, b.n)
    assert ok.all(), f"{(~ok).sum()} quartets outside the gate"


def test_light_ket_and_orientation_agree(lib, h2o26):
    b, q, pre, ref = h2o26
    light, lk = _host_eri(lib, b, q, mode=0)
    full, _ = _host_eri(lib, b, q, mode=1)
    swapped, _ = _host_eri(lib, b, q, mode=2)
    assert (lk < 3).sum() > 0
    assert _gate(light, full, pre, q, b.n).all()
    assert _gate(swapped, full, pre, q, b.n).all()


def test_folding_is_exact(lib):
    """Folding the (m1, m2) / (m2, m1) pairs of same-fit functions changes only the summation
    order: the values agree with the unfolded sum to rounding (1e-14 relative)."""
    b = configs.h2o_minimal(ng0=6)
    q = basis.build_mapping(b.n)
    f, _ = _host_eri(lib, b, q, fold=1)
    u, _ = _host_eri(lib, b, q, fold=0)
    big = np.abs(u) > 1e-12 * np.abs(u).max()
    assert np.max(np.abs(f[big] - u[big]) / np.abs(u[big])) < 1e-13


def _fp32_error(lib, b, q, pre):
    qq = [np.ascontiguousarray(x, np.int32) for x in q]
    out = np.zeros(7)
    assert lib.ss_host_fp32_error(int(b.n), int(b.ld), *eri_host.basis_arrays(b), len(qq[0]), *qq,
                                  np.ascontiguousarray(pre, np.float64), PRIM_FP32_EPS, out) == 0
    return {"n_tier": int(out[3]), "signed": out[4], "abs": out[5], "acc": out[6]}


def test_fp32_tier_error_is_negligible(lib, h2o26):
    """The FP32 tier (primitive quartets below 1e-11 of the Schwarz bound sqrt((ik|ik)(jl|jl)),
    evaluated as the kernel does: FP32 bra polynomials from the FP32 pair copies, ket polynomials
    rounded from FP64, K_AB c folded into the FP32 factor) changes each ERI by far less than the
    1e-12 gate: the sum of |FP32 - FP64| over a quartet's tier, and the rounding of the
    per-thread FP32 running sums, stay below 2e-14 of its Schwarz bound (measured: 1.2e-15 and
    5.0e-15 at 20-Gaussian fits).  (A single primitive quartet can be off by its whole bound when
    its FP32 prefactor underflows, but such terms are ~1e-40 in absolute size.)  Every quartet of
    the 26-function basis at 3-Gaussian fits, and 10 quartets at the production 20-Gaussian fits."""
    from oracle import binding as O
    b, q, pre, ref = h2o26
    e = _fp32_error(lib, b, q, pre)
    assert e["n_tier"] > 0 and e["abs"] < 2e-14
    b20 = configs.h2o_26(ng0=20)
    q20 = np.array(basis.build_mapping(b20.n))
    sel = np.random.default_rng(11).choice(q20.shape[1], 10, replace=False)
    qs = q20[:, sel]
    # the Schwarz diagonal entries these quartets need, from the oracle
    pairs = sorted({(int(i), int(k)) for i, k in zip(qs[0], qs[2])} | {(int(j), int(l)) for j, l in zip(qs[1], qs[3])})
    pq = [np.array([p[0] for p in pairs]), np.array([p[0] for p in pairs]),
          np.array([p[1] for p in pairs]), np.array([p[1] for p in pairs])]
    diag, _ = O.gauss_eri(O.OracleBasis(b20), pq)
    pre20 = np.zeros((b20.n, b20.n))
    for (i, k), v in zip(pairs, diag):
        pre20[i - 1, k - 1] = pre20[k - 1, i - 1] = v
    e20 = _fp32_error(lib, b20, [qs[r] for r in range(4)], pre20.reshape(-1, order="F"))
    assert e20["n_tier"] > 100000 and e20["abs"] < 2e-14
    assert e20["acc"] < 2e-14  # the per-thread FP32 running sums


def test_threshold_matches_the_kernel():
    """The FP32-tier threshold used above is the kernel's (csrc/ss_common.cuh)."""
    import re
    src = (CSRC / "ss_common.cuh").read_text()
    m = re.search(r"constexpr double PRIM_FP32_EPS = ([0-9.eE+-]+);", src)
    assert m and float(m.group(1)) == PRIM_FP32_EPS


SAN_SCRIPT = r"""
import sys, ctypes as C, numpy as np
sys.path.insert(0, sys.argv[1])
from slater_stoch_gb300 import basis, configs
L = C.CDLL(sys.argv[2])
f64p = np.ctypeslib.ndpointer(np.float64, flags="C"); i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
L.ss_host_eri.argtypes = [C.c_int, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, f64p, f64p, C.c_int64,
                          i32p, i32p, i32p, i32p, C.c_int, C.c_int, f64p, i32p]
b = configs.h2o_26(ng0=1); q = basis.build_mapping(b.n)
arrs = [np.ascontiguousarray(b.center, np.float64).reshape(-1), np.ascontiguousarray(b.npower, np.int32).reshape(-1),
        np.ascontiguousarray(b.n_sto, np.int32), np.ascontiguousarray(b.i_type, np.int32),
        np.ascontiguousarray(b.n_gauss, np.int32), np.ascontiguousarray(b.c_gauss, np.float64).reshape(-1),
        np.ascontiguousarray(b.g_gauss, np.float64).reshape(-1), np.ascontiguousarray(b.g_slater, np.float64)]
qq = [np.ascontiguousarray(x, np.int32) for x in q]
for mode in (0, 1, 2):
    out = np.zeros(len(qq[0])); lk = np.zeros(len(qq[0]), np.int32)
    assert L.ss_host_eri(int(b.n), int(b.ld), *arrs, len(qq[0]), *qq, mode, 1, out, lk) == 0
# the FP32 templates and boys32 (the FP32 tier), every quartet in the tier's threshold sweep
from oracle import binding as O
pre = np.ascontiguousarray(O.precond(O.OracleBasis(b)))
L.ss_host_fp32_error.argtypes = [C.c_int, C.c_int, f64p, i32p, i32p, i32p, i32p, f64p, f64p, f64p, C.c_int64,
                                 i32p, i32p, i32p, i32p, f64p, C.c_double, f64p]
res = np.zeros(7)
assert L.ss_host_fp32_error(int(b.n), int(b.ld), *arrs, len(qq[0]), *qq, pre, 1e-6, res) == 0
print("sanitized run ok")
"""


def test_kernel_arithmetic_under_asan_ubsan(tmp_path):
    """The kernel's templates (recursion tables, option subsets, light-ket bounds) built for the
    host with AddressSanitizer, UndefinedBehaviorSanitizer and array-bounds checks, run over every
    quartet class of the 26-function basis in all three orientations: no report.  The local
    arrays are the device code's, so this is a bounds check of the kernel's indexing."""
    import os
    import sys
    gxx, nvcc = shutil.which("g++"), shutil.which("nvcc")
    if gxx is None or nvcc is None:
        pytest.skip("g++ or the CUDA headers not available")
    asan = subprocess.run([gxx, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not asan or not Path(asan).exists():
        pytest.skip("libasan not available")
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"
    lib = tmp_path / "liberi_host_san.so"
    subprocess.run([gxx, "-O1", "-g", "-std=c++17", "-ffp-contract=off", "-Wno-unknown-pragmas", "-shared", "-fPIC",
                    "-fsanitize=address,undefined,bounds", "-fno-omit-frame-pointer", f"-I{cuda_inc}", f"-I{CSRC}",
                    str(HERE / "eri_host_shim.cpp"), "-o", str(lib)], check=True)
    env = dict(os.environ, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", SAN_SCRIPT, str(HERE.parent), str(lib)], env=env,
                       capture_output=True, text=True, timeout=900, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "sanitized run ok" in r.stdout
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr
