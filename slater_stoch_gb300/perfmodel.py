"""Work counts of the two-electron path, for roofline reporting.

* primitive quartets: the reference loops over n_gauss(i)*nc(i) x ... x n_gauss(l)*nc(l)
  primitive Gaussian products per (ik|jl) (src/gauss_ijkl.F90:127-150), nc = 3 for the
  r^2-type fits (i_type 2) and 1 otherwise.
* FP64 flops per primitive quartet of the analytic stage (all eri_kernel launches of one
  job, Schwarz diagonal included): FP64 instructions executed (DFMA counted as 2 flops,
  DMUL/DADD as 1) divided by the primitive quartets, from an ncu capture of the H2O
  26-function basis with 6-Gaussian fits (same kernels and angular classes as the 20-Gaussian
  workload).  The capture command and per-class table are in profiles/eri_kernel_h2o26.md.
"""
from __future__ import annotations

import numpy as np

# executed FP64 flops per primitive quartet of the analytic stage (ncu, see module doc)
EXEC_FLOPS_PER_PRIM = 241.5


def _pair_L(b, f1, f2):
    t1 = 2 if b.i_type[f1] == 2 else 0
    t2 = 2 if b.i_type[f2] == 2 else 0
    return int(max(b.npower[f1, ax] + t1 + b.npower[f2, ax] + t2 for ax in range(3)))


def primitive_quartets_by_class(b, quartets):
    """{L: primitive quartets} summed over the quartet list (no K_AB screening)."""
    is_, js, ks, ls = [np.asarray(a) - 1 for a in quartets]
    nc = np.where(np.asarray(b.i_type) == 2, 3, 1) * np.asarray(b.n_gauss)
    n = b.n
    PL = np.zeros((n, n), dtype=int)
    for i in range(n):
        for k in range(n):
            PL[i, k] = _pair_L(b, i, k)
    L = np.maximum(PL[is_, ks], PL[js, ls])
    prims = nc[is_].astype(float) * nc[ks] * nc[js] * nc[ls]
    return {int(c): float(prims[L == c].sum()) for c in np.unique(L)}


def primitive_quartets(b, quartets) -> float:
    return float(sum(primitive_quartets_by_class(b, quartets).values()))


def eri_fp64_flops(b, quartets) -> float:
    """Executed FP64 flops of the analytic stage of one job."""
    return EXEC_FLOPS_PER_PRIM * primitive_quartets(b, quartets)
