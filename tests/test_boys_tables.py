"""Accuracy of the ERI kernel's table-driven Boys function and exponential (csrc/boys.cuh).

The device code is plain IEEE double arithmetic with explicit fma, so a host build of the same
source (tests/boys_host_shim.cpp, g++ with contraction off) reproduces it; it is checked against
40-digit mpmath values:

* exp_neg(x), x in [-80, 0]: within 2 ulp (relative 4.5e-16);
* F_0(T), T >= 1: within 3e-16 relative (T <= 36 from the grid Taylor table, T > 36 the
  reference's sqrt(pi/T)/2);
* F_n(T), 0 < T < 1, n = 0..16 (table Taylor for F_nf, downward recursion below it): within
  1e-15 relative;
* F_n(T), T >= 1, n >= 1: exactly the reference's upward recursion from F_0 and e^-T.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("boys") / "libboys_host.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wno-unknown-pragmas", "-shared",
                    "-fPIC", str(HERE / "boys_host_shim.cpp"), "-o", str(out)], check=True)
    L = C.CDLL(str(out))
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    L.ss_host_boys.argtypes = [dp, C.c_int, C.c_int, dp]
    L.ss_host_exp_neg.argtypes = [dp, C.c_int, dp]
    return L


def _boys_mp(n, T):
    mp.mp.dps = 40
    T = mp.mpf(T)
    if T == 0:
        return mp.mpf(1) / (2 * n + 1)
    return mp.gammainc(n + mp.mpf(1) / 2, 0, T) / (2 * T ** (n + mp.mpf(1) / 2))


def _host_boys(lib, T, nf):
    T = np.ascontiguousarray(T, dtype=np.float64)
    out = np.zeros(len(T) * 17)
    lib.ss_host_boys(T, len(T), nf, out)
    return out.reshape(len(T), 17)


def test_exp_neg_ulp(lib):
    rng = np.random.default_rng(1)
    x = np.concatenate([-rng.uniform(0, 80, 3000), -rng.uniform(0, 1e-3, 200),
                        [0.0, -1e-300, -0.5, -1.0, -np.log(2) / 64, -np.log(2) / 32, -79.999]])
    got = np.zeros_like(x)
    lib.ss_host_exp_neg(x, len(x), got)
    mp.mp.dps = 40
    ref = np.array([float(mp.exp(mp.mpf(v))) for v in x])
    rel = np.abs(got - ref) / ref
    assert rel.max() <= 4.5e-16, rel.max()


def test_boys_f0_large_T(lib):
    rng = np.random.default_rng(2)
    T = np.concatenate([1.0 + rng.uniform(0, 35, 1500), [1.0, 1.0 + 1 / 16, 35.999, 36.0, 36.0001, 50.0, 80.0,
                                                     80.5, 200.0], 1.0 + np.arange(281) / 8 + 1 / 16])
    got = _host_boys(lib, T, 0)[:, 0]
    ref = np.array([float(_boys_mp(0, t)) for t in T])
    rel = np.abs(got - ref) / ref
    assert rel.max() <= 3e-16, (rel.max(), T[rel.argmax()])


@pytest.mark.parametrize("nf", [0, 1, 3, 6, 10, 16])
def test_boys_small_T(lib, nf):
    rng = np.random.default_rng(3 + nf)
    T = np.concatenate([rng.uniform(0, 1, 150), [1e-12, 1 / 32, 1 / 16 + 1 / 32, 0.5, 0.999999, 0.0]])
    got = _host_boys(lib, T, nf)
    for n in range(nf + 1):
        ref = np.array([float(_boys_mp(n, t)) for t in T])
        rel = np.abs(got[:, n] - ref) / ref
        assert rel.max() <= 1e-15, (n, rel.max(), T[rel.argmax()])


def test_boys_upward_recursion_large_T(lib):
    T = np.array([1.0, 1.7, 3.3, 12.0, 35.5, 36.5, 79.0, 85.0])
    got = _host_boys(lib, T, 16)
    e = np.zeros_like(T)
    lib.ss_host_exp_neg(-T, len(T), e)
    e[T > 80.0] = 0.0
    for t in range(len(T)):
        two_rho_inv = 0.5 * (1.0 / np.sqrt(T[t])) ** 2
        rt = (got[t, 0] - e[t]) * two_rho_inv
        di = 3.0
        for n in range(1, 17):
            assert got[t, n] == rt
            rt = (rt * di - e[t]) * two_rho_inv
            di += 2.0


@pytest.mark.parametrize("nf", [0, 4, 9, 16])
def test_boys32(lib, nf):
    """FP32 Boys values (the primitive quartets evaluated in FP32): relative error within 2e-6
    over T in [0, 60] (grid Taylor + downward recursion below 30, asymptotic form above)."""
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    lib.ss_host_boys32.argtypes = [fp, C.c_int, C.c_int, fp]
    rng = np.random.default_rng(7 + nf)
    T = np.concatenate([rng.uniform(0, 60, 120), [0.0, 1e-6, 0.0625, 29.99, 30.0, 30.01]]).astype(np.float32)
    out = np.zeros(len(T) * 17, np.float32)
    lib.ss_host_boys32(T, len(T), nf, out)
    out = out.reshape(len(T), 17)
    for n in range(nf + 1):
        ref = np.array([float(_boys_mp(n, float(t))) for t in T])
        rel = np.abs(out[:, n] - ref) / ref
        assert rel.max() <= 2e-6, (n, rel.max(), T[rel.argmax()])
