"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE: tests/, smoke check and
bench.py's CPU-baseline leg only; the product never imports this module).

Restates the reference's algorithms (scemama/slater_stoch); see ss_oracle.c for
the file:line each function follows.  Parity status: parity unpinned -- the
reference has no golden outputs and cannot be compiled in this environment; the
oracle is checked against analytic known-answer tests only.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C")


class OrcBasis(C.Structure):
    _fields_ = [("n", C.c_int), ("ld", C.c_int), ("center", C.c_void_p), ("npower", C.c_void_p),
                ("n_sto", C.c_void_p), ("i_type", C.c_void_p), ("n_gauss", C.c_void_p),
                ("c_gauss", C.c_void_p), ("g_gauss", C.c_void_p), ("g_slater", C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        # SS_ORACLE_LIB: an alternative build of the same source (the sanitizer test's)
        path = os.environ.get("SS_ORACLE_LIB") or _build.build()
        L = C.CDLL(str(path))
        L.orc_rint_sum.restype = C.c_double
        L.orc_rint_sum.argtypes = [C.c_int, C.c_double, f64p]
        L.orc_rint.restype = C.c_double
        L.orc_rint.argtypes = [C.c_int, C.c_double]
        L.orc_dierfc.restype = C.c_double
        L.orc_dierfc.argtypes = [C.c_double]
        L.orc_bielec_integral.restype = C.c_double
        L.orc_bielec_integral.argtypes = [C.c_double] * 4 + [f64p] * 4 + [i32p] * 4
        L.orc_set_sum_mode.restype = None
        L.orc_set_sum_mode.argtypes = [C.c_int]
        L.orc_gauss_ijkl.restype = C.c_double
        L.orc_gauss_ijkl.argtypes = [C.POINTER(OrcBasis), C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_precond.restype = None
        L.orc_precond.argtypes = [C.POINTER(OrcBasis), f64p, C.c_int]
        L.orc_gauss_eri.restype = C.c_int64
        L.orc_gauss_eri.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p, i32p, i32p, f64p,
                                    f64p, C.c_int]
        L.orc_gauss_list.restype = None
        L.orc_gauss_list.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p, i32p, i32p, f64p, C.c_int]
        L.orc_gauss_list_timed.restype = None
        L.orc_gauss_list_timed.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p, i32p, i32p, f64p, f64p,
                                           C.c_int]
        L.orc_count_primitive_quartets.restype = C.c_double
        L.orc_count_primitive_quartets.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p,
                                                   i32p, i32p]
        L.orc_zvmc_faithful.restype = C.c_int
        L.orc_zvmc_faithful.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p, i32p, i32p,
                                        C.c_double, f64p, f64p, C.c_int, C.c_int64, C.c_int,
                                        f64p, f64p, C.c_void_p, C.c_int]
        L.orc_zvmc_shared.restype = C.c_int
        L.orc_zvmc_shared.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p, i32p, i32p,
                                      f64p, f64p, f64p, C.c_int, C.c_int64, C.c_int, f64p, f64p,
                                      C.c_void_p, C.c_int]
        L.orc_pair_densities.restype = None
        L.orc_pair_densities.argtypes = [C.POINTER(OrcBasis), C.c_int, i32p, i32p, C.c_int64,
                                         f64p, f64p, f64p]
        L.orc_ijkl_slater_xnynzn.restype = C.c_int
        L.orc_ijkl_slater_xnynzn.argtypes = [i32p, i32p, i32p, i32p, f64p, f64p]
        L.orc_monocenter.restype = C.c_int64
        L.orc_monocenter.argtypes = [C.POINTER(OrcBasis), C.c_int64, i32p, i32p, i32p, i32p, f64p, i32p]
        L.orc_one_elect.restype = None
        L.orc_one_elect.argtypes = [C.POINTER(OrcBasis), C.c_int, f64p, f64p, f64p, f64p, f64p]
        _lib = L
    return _lib


class OracleBasis:
    """Keeps the numpy arrays alive while the C struct points at them."""

    def __init__(self, b):
        self.arrs = dict(center=np.ascontiguousarray(b.center, np.float64),
                         npower=np.ascontiguousarray(b.npower, np.int32),
                         n_sto=np.ascontiguousarray(b.n_sto, np.int32),
                         i_type=np.ascontiguousarray(b.i_type, np.int32),
                         n_gauss=np.ascontiguousarray(b.n_gauss, np.int32),
                         c_gauss=np.ascontiguousarray(b.c_gauss, np.float64),
                         g_gauss=np.ascontiguousarray(b.g_gauss, np.float64),
                         g_slater=np.ascontiguousarray(b.g_slater, np.float64))
        a = self.arrs
        self.s = OrcBasis(int(b.n), int(b.ld), *[a[k].ctypes.data for k in
                                                 ("center", "npower", "n_sto", "i_type", "n_gauss",
                                                  "c_gauss", "g_gauss", "g_slater")])
        self.n = int(b.n)


def _threads(t):
    return int(t if t else (os.cpu_count() or 1))


def rint_sum(n, rho, d1):
    return lib().orc_rint_sum(int(n), float(rho), np.ascontiguousarray(d1, np.float64))


def rint(n, rho):
    return lib().orc_rint(int(n), float(rho))


def dierfc(y):
    return lib().orc_dierfc(float(y))


def bielec_integral(alpha, beta, delta, gama, A, B, Cc, D, pA, pB, pC, pD):
    f = lambda v: np.ascontiguousarray(v, np.float64)
    i = lambda v: np.ascontiguousarray(v, np.int32)
    return lib().orc_bielec_integral(alpha, beta, delta, gama, f(A), f(B), f(Cc), f(D), i(pA),
                                     i(pB), i(pC), i(pD))


def set_sum_mode(mode: str):
    """'reference': sequential FP64 sum as src/gauss_ijkl.F90; 'extended': long double sum."""
    lib().orc_set_sum_mode(1 if mode == "extended" else 0)


def gauss_ijkl(ob: OracleBasis, i, k, j, l):
    """0-based (ik|jl) of the fits."""
    return lib().orc_gauss_ijkl(C.byref(ob.s), i, k, j, l)


def precond(ob: OracleBasis, nthreads=0):
    out = np.zeros(ob.n * ob.n)
    lib().orc_precond(C.byref(ob.s), out, _threads(nthreads))
    return out


def gauss_eri(ob: OracleBasis, quartets, pre=None, nthreads=0):
    is_, js, ks, ls = [np.ascontiguousarray(a, np.int32) for a in quartets]
    if pre is None:
        pre = precond(ob, nthreads)
    out = np.zeros(len(is_))
    nz = lib().orc_gauss_eri(C.byref(ob.s), len(is_), is_, js, ks, ls, pre, out, _threads(nthreads))
    return out, int(nz)


def gauss_list(ob: OracleBasis, quartets, nthreads=0):
    """gauss_ijkl of each listed (1-based) quartet, no screening or diagonal shortcut."""
    q = [np.ascontiguousarray(a, np.int32) for a in quartets]
    out = np.zeros(len(q[0]))
    lib().orc_gauss_list(C.byref(ob.s), len(q[0]), *q, out, _threads(nthreads))
    return out


def gauss_list_timed(ob: OracleBasis, quartets, nthreads=0):
    """gauss_list plus each quartet's own seconds on the thread that computed it."""
    q = [np.ascontiguousarray(a, np.int32) for a in quartets]
    out = np.zeros(len(q[0]))
    sec = np.zeros(len(q[0]))
    lib().orc_gauss_list_timed(C.byref(ob.s), len(q[0]), *q, out, sec, _threads(nthreads))
    return out, sec


def count_primitive_quartets(ob: OracleBasis, quartets):
    is_, js, ks, ls = [np.ascontiguousarray(a, np.int32) for a in quartets]
    return lib().orc_count_primitive_quartets(C.byref(ob.s), len(is_), is_, js, ks, ls)


def zvmc_faithful(ob: OracleBasis, quartets, a_zv, r1, r2, nblocks, npts, mode="fp64",
                  return_blocks=False, nthreads=0):
    is_, js, ks, ls = [np.ascontiguousarray(a, np.int32) for a in quartets]
    nint = len(is_)
    mean = np.zeros(nint)
    err = np.zeros(nint)
    xb = np.zeros(nblocks * nint) if return_blocks else None
    rc = lib().orc_zvmc_faithful(C.byref(ob.s), nint, is_, js, ks, ls, float(a_zv),
                                 np.ascontiguousarray(r1, np.float64).reshape(-1),
                                 np.ascontiguousarray(r2, np.float64).reshape(-1), int(nblocks),
                                 int(npts), 0 if mode == "ref32" else 1, mean, err,
                                 xb.ctypes.data if xb is not None else None, _threads(nthreads))
    if rc != 0:
        raise ValueError("npts must be a multiple of 40")
    if return_blocks:
        return mean, err, xb.reshape(nblocks, nint)
    return mean, err


def zvmc_shared(ob: OracleBasis, quartets, u1, u2, w, nblocks, npts, symmetrize=True,
                return_blocks=False, nthreads=0):
    is_, js, ks, ls = [np.ascontiguousarray(a, np.int32) for a in quartets]
    nint = len(is_)
    mean = np.zeros(nint)
    err = np.zeros(nint)
    xb = np.zeros(nblocks * nint) if return_blocks else None
    lib().orc_zvmc_shared(C.byref(ob.s), nint, is_, js, ks, ls,
                          np.ascontiguousarray(u1, np.float64).reshape(-1),
                          np.ascontiguousarray(u2, np.float64).reshape(-1),
                          np.ascontiguousarray(w, np.float64).reshape(-1), int(nblocks), int(npts),
                          1 if symmetrize else 0, mean, err,
                          xb.ctypes.data if xb is not None else None, _threads(nthreads))
    if return_blocks:
        return mean, err, xb.reshape(nblocks, nint)
    return mean, err


def pair_densities(ob: OracleBasis, ip, kp, u):
    ip = np.ascontiguousarray(ip, np.int32)
    kp = np.ascontiguousarray(kp, np.int32)
    u = np.ascontiguousarray(u, np.float64).reshape(-1, 3)
    S = u.shape[0]
    rs = np.zeros((len(ip), S))
    rg = np.zeros((len(ip), S))
    lib().orc_pair_densities(C.byref(ob.s), len(ip), ip, kp, S, u.reshape(-1), rs, rg)
    return rs, rg


def one_elect(ob: OracleBasis, xyz, charge):
    """Overlap, nuclear attraction and kinetic matrices (n x n, [i, k]) of the fits
    (src/one_elect.F90); xyz (nat, 3) bohr, charge (nat,)."""
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
    charge = np.ascontiguousarray(charge, np.float64)
    n = ob.s.n
    S = np.zeros(n * n); V = np.zeros(n * n); K = np.zeros(n * n)
    lib().orc_one_elect(C.byref(ob.s), len(charge), xyz, charge, S, V, K)
    return (S.reshape(n, n, order="F"), V.reshape(n, n, order="F"), K.reshape(n, n, order="F"))


def ijkl_slater_xnynzn(nix, niy, niz, power, gamma):
    """Exact one-centre Slater ERI (1 2|3 4) of x^nx y^ny z^nz r^power e^(-gamma r) functions
    (src/ijkl_slater_xnynzn.F90)."""
    a = [np.ascontiguousarray(x, np.int32) for x in (nix, niy, niz, power)]
    out = np.zeros(1)
    rc = lib().orc_ijkl_slater_xnynzn(*a, np.ascontiguousarray(gamma, np.float64), out)
    if rc:
        raise ValueError("x^nx y^ny z^nz Slater functions beyond d are not implemented (as the reference)")
    return float(out[0])


def monocenter(ob: OracleBasis, quartets):
    """Exact values of the one-centre quartets (src/two_e_slater.F90:318-369): (values, mask);
    values are 0 where mask is 0."""
    q = [np.ascontiguousarray(x, np.int32) for x in quartets]
    out = np.zeros(len(q[0]))
    mask = np.zeros(len(q[0]), np.int32)
    cnt = lib().orc_monocenter(C.byref(ob.s), len(q[0]), *q, out, mask)
    if cnt < 0:
        raise ValueError("one-centre quartet with a function beyond d (not implemented, as the reference)")
    return out, mask.astype(bool)
