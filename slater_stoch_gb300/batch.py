"""Many systems of uneven size in one analytic launch per kernel class (the batched workload).

The reference runs one system per process (src/two_e_slater.F90:219-564).  Here the systems'
fitted bases are concatenated into one basis, ``ss_basis_systems`` marks the system boundaries
(primitive pairs of functions of two systems are never formed), and the systems' own unique
quartet lists, concatenated with their function indices shifted, go to one ``ss_gauss_eri``:
the analytic stage of every system then runs as one launch per kernel instance (L, LK, tc),
quartets of all systems mixed, which fills the GPU where a small system alone would leave most
SMs idle.  The ZV-MC correction of each system runs as its own job on the pooled worker
contexts (``SS_JOB_MC_ONLY``: its proposal mixture is the system's own), all of them
concurrently; each system's ERIs are its analytic values plus its correction.

A system's result does not depend on the batch it ran in beyond summation order: the analytic
values agree with a run of the system alone to rounding (the bra-slice split of a quartet
depends on how many quartets share its kernel class), and the MC correction is bitwise the
same (same seed, same walkers, same reductions).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import api, basis
from ._lib import check


def concat_systems(systems):
    """(combined Basis, first function of each system (1-based, nsys+1 entries))."""
    ld = max(b.ld for b in systems)
    n = sum(b.n for b in systems)
    out = basis.Basis(center=np.zeros((n, 3)), npower=np.zeros((n, 3), np.int32),
                      n_sto=np.zeros(n, np.int32), i_type=np.zeros(n, np.int32),
                      n_gauss=np.zeros(n, np.int32), c_gauss=np.zeros((2, n, ld)),
                      g_gauss=np.zeros((n, ld)), g_slater=np.zeros(n), nucleus=np.zeros(n, np.int32),
                      names=[], shell=np.zeros(n, np.int32))
    first = [1]
    o = 0
    for b in systems:
        m = b.n
        out.center[o:o + m] = b.center
        out.npower[o:o + m] = b.npower
        out.n_sto[o:o + m] = b.n_sto
        out.i_type[o:o + m] = b.i_type
        out.n_gauss[o:o + m] = b.n_gauss
        out.c_gauss[:, o:o + m, :b.ld] = b.c_gauss
        out.g_gauss[o:o + m, :b.ld] = b.g_gauss
        out.g_slater[o:o + m] = b.g_slater
        out.nucleus[o:o + m] = b.nucleus
        out.names += list(b.names)
        out.shell[o:o + m] = b.shell
        o += m
        first.append(o + 1)
    return out, np.array(first, dtype=np.int32)


@dataclass
class BatchReport:
    nsys: int
    nbasis: list
    unique_eris: int
    analytic_s: float = 0.0
    wall_s: float = 0.0
    latency_s: list = field(default_factory=list)   # per system: batch start -> its result ready
    blocks: list = field(default_factory=list)
    max_sigma: list = field(default_factory=list)

    def summary(self) -> dict:
        lat = np.sort(np.asarray(self.latency_s))
        pct = lambda p: float(lat[min(len(lat) - 1, int(np.ceil(p * len(lat))) - 1)])
        return {"systems": self.nsys, "nbasis_min_max": [int(min(self.nbasis)), int(max(self.nbasis))],
                "unique_eris": self.unique_eris, "analytic_s": self.analytic_s, "wall_s": self.wall_s,
                "eris_per_s": self.unique_eris / self.wall_s if self.wall_s > 0 else None,
                "p50_ms": 1e3 * pct(0.5), "p99_ms": 1e3 * pct(0.99),
                "max_sigma_Ha": float(max(self.max_sigma)) if self.max_sigma else None,
                "mean_blocks": float(np.mean(self.blocks)) if self.blocks else None}


def batch_two_e(systems, seeds, sigma_target: float = 1e-6, npts: int = 1 << 16, nblocks_max: int = 64,
                a_zv: float = 1.8, device: int = 0, max_running: int = 8):
    """ERIs and error bars of every system; returns (list of (eri, sigma), BatchReport)."""
    comb, first = concat_systems(systems)
    qs, offs = [], [0]
    for s, b in enumerate(systems):
        q = basis.build_mapping(b.n)
        sh = int(first[s]) - 1
        qs.append([np.asarray(x, np.int32) + sh for x in q])
        offs.append(offs[-1] + len(q[0]))
    cat = [np.ascontiguousarray(np.concatenate([q[c] for q in qs])) for c in range(4)]
    rep = BatchReport(nsys=len(systems), nbasis=[b.n for b in systems], unique_eris=offs[-1])
    results = [None] * len(systems)
    with api.Context(device) as ctx:
        t0 = time.perf_counter()
        ctx.set_basis(comb)
        check(ctx._L.ss_basis_systems(ctx._h, len(systems), first))
        ctx.set_quartets(*cat)
        ctx.job_limits(0, max_running)
        # the MC jobs first (they run on the worker contexts while the analytic stage runs here)
        jids = [ctx.job_submit_inputs(b, basis.build_mapping(b.n), a_zv, int(sd), npts, nblocks_max,
                                      "shared", "split_bf16", sigma_target, mc_only=True)
                for b, sd in zip(systems, seeds)]
        g, _ = ctx.gauss_eri()
        rep.analytic_s = time.perf_counter() - t0
        pending = dict(enumerate(jids))
        while pending:
            for s, jid in list(pending.items()):
                if ctx.job_poll(jid):
                    info = ctx.job_info(jid)
                    mean, sig = ctx.job_result(jid)
                    gs = g[offs[s]:offs[s + 1]]
                    results[s] = (gs + mean, sig)
                    rep.latency_s.append(max(time.perf_counter() - t0, rep.analytic_s))
                    rep.blocks.append(info["blocks"])
                    rep.max_sigma.append(info["max_sigma"])
                    del pending[s]
            time.sleep(0.0005)
        rep.wall_s = time.perf_counter() - t0
    return results, rep
