"""Work counts of the two-electron path, for roofline reporting.

* primitive quartets: the reference loops over n_gauss(i)*nc(i) x ... x n_gauss(l)*nc(l)
  primitive Gaussian products per (ik|jl) (src/gauss_ijkl.F90:127-150), nc = 3 for the
  r^2-type fits (i_type 2) and 1 otherwise.  The GPU skips the primitive quartets below its
  Schwarz screen and evaluates those below the FP32 bound in FP32, so the executed work is
  measured rather than modelled:
* EXEC_FLOPS: executed flops of all eri_kernel launches of one job (Schwarz factors, Schwarz
  diagonal and screened quartets), from ncu instruction counters on the full workload
  (smsp__sass_thread_inst_executed_op_{dfma,dmul,dadd,ffma}_pred_on.sum, one pass each; DFMA
  and FFMA counted as 2 flops), and EXEC_DRAM_BYTES their DRAM traffic (the per-class table and
  the command are kept with the profiles).
* EXEC_FLOPS_PER_PRIM: the earlier all-FP64 kernel's executed FP64 flops per primitive quartet
  (241.5, unscreened), kept as the model for workloads without a measurement.
"""
from __future__ import annotations

import numpy as np

# executed FP64 flops per primitive quartet of the all-FP64 kernel (fallback model)
EXEC_FLOPS_PER_PRIM = 241.5

# workload -> (executed FP64 flops, executed FP32 FFMA flops) of the analytic stage of one job, at
# the default tiers (primitive screen 1e-18, FP32 tier below 1e-11 of the Schwarz bound)
EXEC_FLOPS = {
    "h2o_26_ng20": (5.518e11, 4.700e11),
}
# workload -> DRAM bytes (read + write) of all eri_kernel launches of one job (ncu
# dram__bytes_read.sum + dram__bytes_write.sum, one pass each; mostly the local-memory spill
# traffic of the L = 4 classes with several r^2-type fits)
# workload -> DRAM bytes per walker pair of the shared-walker MC kernels (sampler, orbital values,
# operands, tcgen05 GEMM, accumulation): ncu --set full of one 262,144-sample sub-chunk (reads
# 2.0146e9 B + writes 1.5291e9 B) / 262,144
MC_DRAM_BYTES_PER_SAMPLE = {
    "h2o_26_ng20": 3.5437e9 / 262144,
}
EXEC_DRAM_BYTES = {
    "h2o_26_ng20": 1.2443e10,
}


def _pair_L(b, f1, f2):
    t1 = 2 if b.i_type[f1] == 2 else 0
    t2 = 2 if b.i_type[f2] == 2 else 0
    return int(max(b.npower[f1, ax] + t1 + b.npower[f2, ax] + t2 for ax in range(3)))


def kernel_classes(b, quartets):
    """The analytic kernel instance (L, LK, tc) of every quartet, as the device buckets them:
    L = the larger pair's per-axis degree bound, tc = the number of r^2-type fits among the four
    functions, LK = the lighter pair's bound lmin for lmin < L <= 3, max(lmin, 1) for L = 4 and
    lmin <= 2, else L.  Returns an (nq, 3) int array."""
    is_, js, ks, ls = [np.asarray(a) - 1 for a in quartets]
    n = b.n
    PL = np.zeros((n, n), dtype=np.int64)
    for i in range(n):
        for k in range(n):
            PL[i, k] = _pair_L(b, i, k)
    Lb, Lk = PL[is_, ks], PL[js, ls]
    L = np.maximum(Lb, Lk)
    lmin = np.minimum(Lb, Lk)
    r2 = (np.asarray(b.i_type) == 2).astype(np.int64)
    tc = r2[is_] + r2[ks] + r2[js] + r2[ls]
    # the light-ket rule of ss_light_ket (csrc/ss_common.cuh)
    LK = np.where(lmin >= L, L, np.where(L == 4, np.where(lmin <= 2, np.maximum(lmin, 1), L), lmin))
    return np.stack([L, LK, tc], axis=1)


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


def eri_fp64_flops(b, quartets, workload: str | None = None) -> float:
    """Executed FP64 flops of the analytic stage of one job: the ncu measurement when the
    workload has one, else the all-FP64 model."""
    if workload in EXEC_FLOPS:
        return EXEC_FLOPS[workload][0]
    return EXEC_FLOPS_PER_PRIM * primitive_quartets(b, quartets)
