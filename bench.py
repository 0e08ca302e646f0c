"""Benchmark of the two-electron ZV-MC path on one GB300 (or N replicas).

Workload (default): H2O, 26-function STO basis, 20-Gaussian fits, all 61,776 unique (ik|jl),
2^26 walker pairs; one step = the reference driver's whole job (src/two_e_slater.F90:219-564):
Schwarz diagonal + analytic Gaussian-fit ERIs (FP64) + ZV-MC correction (shared-walker
estimator, split-BF16 tcgen05 contraction) + merge.  Metric: unique ERIs per second of job
wall time, with the job's largest MC error reported (target sigma <= 1e-6 Ha).

Also measured: the same GPU's FP64 plain path (faithful per-pair estimator in FP64; its MC cost
is exactly proportional to the walker count, so it is timed on a bounded walker sample and
scaled), and the CPU oracle (restated reference algorithm, all host cores) on a bounded sample.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NINT_WORKLOAD = "h2o_26"
METRIC = "unique ERIs/s at sigma<=1e-6 Ha (two-electron ZV-MC job), split-BF16 vs FP64 plain"
WORKLOAD = ("h2o_26: H2O O(0,0,0) H(0,+-1.4305,1.1093) bohr, 26 STOs, 20-Gaussian fits, "
            "61776 unique ERIs, 2^26 walker pairs")
WALKERS = 1 << 26
NBLOCKS = 16
A_ZV = 1.8
SIGMA_TARGET = 1e-6


def _workload():
    from slater_stoch_gb300 import basis, configs
    b = configs.h2o_26(ng0=20)
    q = basis.build_mapping(b.n)
    return b, q


# ------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ------------------------------------------------------------------------------------------
# CPU baseline: the oracle (restated reference) on bounded samples of the workload
# ------------------------------------------------------------------------------------------
def _class_keys(b, quartets):
    from slater_stoch_gb300.perfmodel import kernel_classes
    c = kernel_classes(b, quartets)
    return c[:, 0] * 100 + c[:, 1] * 10 + c[:, 2]


def _sampled_seconds(O, ob, quartets, keys, rng, per_class, cores):
    """Estimated wall seconds of gauss_ijkl over every listed quartet on `cores` threads: a sample
    stratified by kernel class (L, LK, tc) runs on all threads at once, each quartet timed on the
    thread that computed it, and each class's sampled seconds are scaled by the class's
    primitive-quartet count (the cost per primitive quartet differs several-fold between
    classes; the quartets are independent, so the job divides over the cores)."""
    qa = [np.asarray(a) for a in quartets]
    sel = []
    for key in np.unique(keys):
        idx = np.nonzero(keys == key)[0]
        sel.extend(rng.choice(idx, min(per_class, idx.size), replace=False).tolist())
    sel = np.array(sorted(sel))
    _, sec = O.gauss_list_timed(ob, [np.ascontiguousarray(a[sel]) for a in qa], cores)
    total, sub_all, all_all = 0.0, 0.0, 0.0
    for key in np.unique(keys):
        idx = np.nonzero(keys == key)[0]
        m = keys[sel] == key
        cls_prims = O.count_primitive_quartets(ob, [np.ascontiguousarray(a[idx]) for a in qa])
        sub_prims = O.count_primitive_quartets(ob, [np.ascontiguousarray(a[sel[m]]) for a in qa])
        total += sec[m].sum() * cls_prims / max(sub_prims, 1.0)
        sub_all += sub_prims
        all_all += cls_prims
    return total / cores, len(sel), sub_all, all_all


def cpu_baseline(b, q, seed: int = 0, per_class: int = 4):
    """One bounded sample of the job on the host cores, scaled to the whole job: the Schwarz
    diagonal and the unique quartets each from a sample stratified by kernel class, the faithful
    ZV-MC on 4,000 walkers (its cost is exactly proportional to the walker count)."""
    from oracle import binding as O
    ob = O.OracleBasis(b)
    nint = len(q[0])
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    n = b.n
    di = np.array([i for i in range(1, n + 1) for k in range(1, i + 1)], np.int32)
    dk = np.array([k for i in range(1, n + 1) for k in range(1, i + 1)], np.int32)
    dq = [di, di, dk, dk]
    t_pre, n_pre, _, _ = _sampled_seconds(O, ob, dq, _class_keys(b, dq), rng, max(per_class - 1, 1), cores)
    t_eri, n_eri, sub_prims, total_prims = _sampled_seconds(O, ob, q, _class_keys(b, q), rng, per_class, cores)
    npts = 40 * 100
    r = np.random.default_rng(1000 + seed)
    r1 = r.standard_normal((npts, 3))
    r2 = r.standard_normal((npts, 3))
    t = time.perf_counter()
    O.zvmc_faithful(ob, q, A_ZV, r1, r2, 1, npts, "ref32", nthreads=cores)
    t_mc_sample = time.perf_counter() - t
    t_mc = t_mc_sample * WALKERS / npts
    t_analytic = t_pre + t_eri
    job = t_analytic + t_mc
    return {
        "value": nint / job, "unit": "ERIs/s", "cores": cores, "kind": "port",
        "sample": (f"oracle (C restatement of the reference, OpenMP {cores} threads): Schwarz diagonal from "
                   f"{n_pre} and unique quartets from {n_eri} quartets stratified by kernel class ({sub_prims:.3g} "
                   f"of {total_prims:.3g} primitive quartets), each quartet timed on its thread and each class "
                   f"scaled by its primitive-quartet count ({t_analytic:.0f} s estimated on {cores} cores); "
                   f"faithful ZV-MC (ref32 casts) on {npts} walkers ({t_mc_sample:.2f} s) scaled to {WALKERS}"),
        "job_seconds_estimated": job, "analytic_s": t_analytic, "mc_s": t_mc,
    }


def run_reference(args):
    """The reference's algorithm on the host cores (the C oracle restatement, OpenMP on all
    cores; the Fortran reference cannot be built here).  Each step is one bounded sample of the
    job (Schwarz-diagonal and unique quartets stratified by kernel class, 4,000 faithful walkers)
    scaled to the whole job, a different sample each step; W untimed steps, then K timed ones;
    value = ERIs per estimated job second."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    b, q = _workload()
    for w in range(args.warmup):
        cpu_baseline(b, q, seed=1000 + w, per_class=2)
    steps = [cpu_baseline(b, q, seed=s, per_class=2) for s in range(max(args.steps, 1))]
    job_s = statistics.mean(c["job_seconds_estimated"] for c in steps)
    nint = len(q[0])
    value = nint / job_s
    cb = steps[-1]
    line = {
        "impl": "reference", "metric": METRIC,
        "value": value, "unit": "ERIs/s", "n_gpus": args.gpus, "steps": len(steps), "warmup": args.warmup,
        "ms_per_step": job_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (ref32 casts in the MC)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "walkers": WALKERS, "blocks": NBLOCKS,
                   "estimator": "faithful (the reference's per-pair ZV map), ref32 casts",
                   "parallelism": f"host, {cb['cores']} threads"},
        "cpu_baseline": {"value": value, "unit": "ERIs/s", "cores": cb["cores"], "kind": cb["kind"],
                         "sample": cb["sample"]},
        "e2e": {"value": value, "unit": "ERIs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def serving_run(rate: float, duration: float, large: str, max_running: int, seed: int = 1,
                max_atoms: int = 1) -> dict:
    """Open-loop Poisson serving run (slater_stoch_gb300.serving): requests arrive at `rate`
    per second for `duration` seconds, each a small random system (1..max_atoms atoms of the
    random-molecule rules: 4 or 11 STOs for one atom) or with probability 0.05 the `large`
    system, with error-bar targets log-uniform in [1e-7, 1e-5] Ha; admitted within a 150 GB ERI
    budget and `max_running` concurrent jobs, each retired at its target."""
    from slater_stoch_gb300 import configs, serving
    big = getattr(configs, large)(ng0=20)
    reqs = serving.make_requests(seed, rate, duration, large=big, max_atoms=max_atoms)
    t = time.perf_counter()
    rep = serving.serve(reqs, max_running=max_running)
    out = rep.summary()
    out.update({"rate_per_s": rate, "duration_s": duration, "large_system": large, "max_atoms": max_atoms,
                "requests": len(reqs), "max_running": max_running,
                "sizes_nbasis": [int(min(r.basis.n for r in reqs)), int(max(r.basis.n for r in reqs))],
                "elapsed_s": time.perf_counter() - t})
    return out


def batch_run(nsys: int, min_atoms: int, max_atoms: int, seed: int = 1, max_running: int = 8) -> dict:
    """The batched workload: `nsys` seeded systems of the random-molecule rules with min..max
    atoms (uneven sizes) in one basis, their analytic ERIs in one launch per kernel class, each
    system's MC (to max sigma <= 1e-6 Ha) as its own concurrent job; latency of a system = batch
    start to its result."""
    from slater_stoch_gb300 import batch, configs
    rng = np.random.default_rng(seed)
    systems = [configs.random_molecule(int(rng.integers(1, 2 ** 31 - 1)),
                                       natoms=int(rng.integers(min_atoms, max_atoms + 1)), box=4.0)
               for _ in range(nsys)]
    _, rep = batch.batch_two_e(systems, list(range(1, nsys + 1)), sigma_target=SIGMA_TARGET,
                               max_running=max_running)
    out = rep.summary()
    out.update({"atoms_per_system": [min_atoms, max_atoms]})
    return out


def random_molecule_run(natoms: int, mol_seed: int, seed: int, rank: int, q: int) -> dict:
    """The large single-system workload: the seeded random molecule (12 atoms: 111 STOs,
    1.93e7 unique ERIs), one job to max sigma <= 1e-6 Ha (shared-walker split-BF16 estimator,
    blocks of 2^20 walker pairs, at most 256 blocks = 2^28), timed with CUDA events on the
    library stream, then the randomized-SVD cleanup (rank `rank`, q power iterations) of the
    packed pair metric."""
    import torch
    from slater_stoch_gb300 import api, basis, configs
    b = configs.random_molecule(mol_seed, natoms=natoms)
    qq = basis.build_mapping(b.n)
    nint = len(qq[0])
    npts, nmax = 1 << 20, 256
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*qq)
        st = torch.cuda.ExternalStream(ctx.stream_ptr)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        ctx.gauss_eri(copy=False)
        e1.record(st)
        ctx.zvmc(A_ZV, seed, npts, nmax, "shared", "split_bf16", SIGMA_TARGET, copy=False)
        e2.record(st)
        e2.synchronize()
        t_an, t_mc = e0.elapsed_time(e1) * 1e-3, e1.elapsed_time(e2) * 1e-3
        out = {"natoms": natoms, "mol_seed": mol_seed, "nbasis": b.n, "unique_eris": nint,
               "analytic_s": t_an, "mc_s": t_mc, "eris_per_s": nint / (t_an + t_mc),
               "max_sigma_Ha": ctx.max_sigma, "blocks": ctx.blocks_done, "walkers": ctx.blocks_done * npts,
               "sigma_target_Ha": SIGMA_TARGET}
        eri = ctx.combine()
        out["nonfinite_eris"] = int((~np.isfinite(eri)).sum())
        try:
            t = time.perf_counter()
            _, nrem = ctx.psd_clean(eri, layout="packed_pair", rank=rank, oversample=0, q=q, seed=seed)
            out.update({"svd_clean_s": time.perf_counter() - t, "svd_clean_removed": nrem,
                        "svd_clean": f"packed pair metric N={b.n * (b.n + 1) // 2}, rank {rank}, q {q}, FP64"})
        except Exception as ex:
            out["svd_clean_error"] = str(ex)
    return out


def fp64_peak_tflops(torch):
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    bm = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, bm)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(3):
        e0.record()
        torch.matmul(a, bm)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--walkers", type=int, default=WALKERS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="h2o_26", choices=["h2o_26", "serve", "random", "batch"],
                    help="serve: only the open-loop serving run; random: only the large random-molecule "
                         "job (each its own JSON line)")
    ap.add_argument("--natoms", type=int, default=12, help="random: atoms of the random molecule")
    ap.add_argument("--systems", type=int, default=64, help="batch: number of systems")
    ap.add_argument("--atoms", type=int, nargs=2, default=[1, 3], help="batch: min and max atoms per system")
    ap.add_argument("--mol-seed", type=int, default=1, help="random: seed of the random molecule")
    ap.add_argument("--rate", type=float, default=15.0, help="serving: arrivals per second")
    ap.add_argument("--duration", type=float, default=20.0, help="serving: seconds of arrivals")
    ap.add_argument("--large", default="h2o_minimal", help="serving: the 5%% large system")
    ap.add_argument("--max-running", type=int, default=8, help="serving: concurrent jobs")
    ap.add_argument("--max-atoms", type=int, default=1, help="serving: atoms per small system")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-cleanup", action="store_true", help="skip the cleanup section (profiling runs)")
    ap.add_argument("--fp32-eps", type=float, default=None,
                    help="FP32-tier threshold of the analytic stage (ss_set_eri_tiers); default: the library's")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "random":
        line = {"metric": "unique ERIs/s at sigma<=1e-6 Ha, one large system (seeded random molecule)",
                "workload": "random", "random": random_molecule_run(args.natoms, args.mol_seed, 1, 512, 4)}
        print(json.dumps(line))
        return
    if args.workload == "batch":
        line = {"metric": "unique ERIs/s and per-system p50/p99 latency, many systems in one batched launch",
                "workload": "batch", "batch": batch_run(args.systems, args.atoms[0], args.atoms[1],
                                                        max_running=args.max_running)}
        print(json.dumps(line))
        return
    if args.workload == "serve":
        line = {"metric": "unique ERIs/s under open-loop Poisson arrivals; p50/p99 job latency",
                "workload": "serve", "serving": serving_run(args.rate, args.duration, args.large, args.max_running,
                                               max_atoms=args.max_atoms)}
        print(json.dumps(line))
        return

    import torch
    import torch.distributed as dist
    from slater_stoch_gb300 import api
    from slater_stoch_gb300.perfmodel import eri_fp64_flops
    from slater_stoch_gb300.replicas import job_seed, max_over_ranks, whole_job_throughput

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    b, q = _workload()
    nint = len(q[0])
    npts = args.walkers // NBLOCKS
    ctx = api.Context(local)
    ctx.set_basis(b)
    ctx.set_quartets(*q)
    if args.fp32_eps is not None:
        ctx.set_eri_tiers(1e-18, args.fp32_eps)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    seed = job_seed(1, rank)

    def job():
        ctx.two_e_job(A_ZV, seed, npts, NBLOCKS, "shared", "split_bf16", 0.0, copy=False)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        job()
    barrier()
    times = []
    l0 = ctx.launches
    with ClockSampler(local) as clk:
        barrier()
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.nvtx.range_push("timed_job")  # ncu --nvtx-include "timed_job/" selects these launches
            e0.record(stream)
            job()
            e1.record(stream)
            e1.synchronize()
            torch.cuda.nvtx.range_pop()
            times.append(e0.elapsed_time(e1))
        barrier()
        t_wall = time.perf_counter() - t_wall0
    launches = (ctx.launches - l0) // max(args.steps, 1)
    max_sigma = ctx.max_sigma
    ms_step = max_over_ranks(sum(times), world, dist, dev) / args.steps
    value = whole_job_throughput(nint, world, ms_step * 1e-3)

    # end-to-end through the C ABI with host buffers: upload basis + quartets, copy results back
    e2e_times = []
    for _ in range(max(1, min(args.steps, 2))):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        c2 = api.Context(local)
        c2.set_basis(b)
        c2.set_quartets(*q)
        if args.fp32_eps is not None:
            c2.set_eri_tiers(1e-18, args.fp32_eps)
        eri, sig = c2.two_e_job(A_ZV, seed, npts, NBLOCKS, "shared", "split_bf16", 0.0, copy=True)
        e2e_times.append(time.perf_counter() - t)
        c2.close()
    e2e_s = max_over_ranks(statistics.median(e2e_times), world, dist, dev)  # the slowest rank's job
    h2d = sum(a.nbytes for a in ctx._basis_arrays) + 4 * 4 * nint
    d2h = 2 * 8 * nint

    # stage split of one job (events on the library stream)
    ctx.invalidate()
    torch.cuda.synchronize()
    s0, s1, s2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    s0.record(stream)
    ctx.gauss_eri(copy=False)
    s1.record(stream)
    ctx.zvmc(A_ZV, seed, npts, NBLOCKS, "shared", "split_bf16", copy=False)
    s2.record(stream)
    s2.synchronize()
    t_analytic = s0.elapsed_time(s1) * 1e-3
    t_mc = s1.elapsed_time(s2) * 1e-3

    # cleanup of the final ERIs (host arrays through the C ABI): randomized-SVD svd_clean on the
    # packed 351x351 metric (rank 200, oversampling 10, 4 power iterations), the exact projection
    # of the remaining negative components, and Davidson for the lowest 10 eigenpairs
    eri_final, _ = ctx.two_e_job(A_ZV, seed, npts, NBLOCKS, "shared", "split_bf16", 0.0, copy=True)
    cleanup = {"nonfinite_eris": int((~np.isfinite(eri_final)).sum())}
    try:  # reported, not fatal for the throughput line
        if args.no_cleanup:
            raise RuntimeError("skipped (--no-cleanup)")
        t = time.perf_counter()
        c1, n_svd = ctx.psd_clean(eri_final, layout="packed_pair", rank=200, oversample=10, q=4, seed=seed)
        t_svd = time.perf_counter() - t
        t = time.perf_counter()
        c2, n_proj = ctx.psd_project(c1, layout="packed_pair")
        t_proj = time.perf_counter() - t
        cleanup.update({"svd_clean_s": t_svd, "svd_clean_removed": n_svd, "project_s": t_proj,
                        "project_removed": n_proj,
                        "value_with_cleanup": world * nint / (ms_step * 1e-3 + t_svd + t_proj)})
        t = time.perf_counter()
        dav_ev, _ = ctx.davidson(c2, m=10, layout="packed_pair", tol=1e-6, max_iter=5000)
        cleanup.update({"davidson_s": time.perf_counter() - t,
                        "davidson_lowest10_Ha": [float(v) for v in dav_ev]})
    except Exception as ex:
        cleanup["error"] = str(ex)

    # FP64 plain path: faithful per-pair estimator in FP64; MC time is linear in walkers
    plain_npts = 40 * 8192
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.zvmc(A_ZV, seed, 40 * 256, 1, "faithful", "fp64", copy=False)  # warm
    p0.record(stream)
    ctx.zvmc(A_ZV, seed, plain_npts, 1, "faithful", "fp64", copy=False)
    p1.record(stream)
    p1.synchronize()
    t_plain_mc = p0.elapsed_time(p1) * 1e-3 * args.walkers / plain_npts
    plain_value = nint / (t_analytic + t_plain_mc)

    from slater_stoch_gb300.perfmodel import primitive_quartets
    nprim = primitive_quartets(b, q)
    from slater_stoch_gb300.perfmodel import EXEC_DRAM_BYTES, EXEC_FLOPS
    wl = f"{NINT_WORKLOAD}_ng20"
    flops = eri_fp64_flops(b, q, wl)
    peak64 = fp64_peak_tflops(torch)
    achieved = flops / t_analytic / 1e12 if flops else None
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                "frac": achieved / peak64 if (peak64 and achieved) else None,
                "traffic": EXEC_DRAM_BYTES.get(wl),
                "traffic_note": "DRAM bytes of all eri_kernel launches of one job (ncu, one pass per metric)",
                "kernel": "eri_kernel (analytic Gaussian-fit ERIs, all launches of one job)",
                "peak_source": "measured in this run: torch float64 matmul 4096^3 (FP64 peak is not "
                               "in MEASURED_PEAKS.json)",
                "fp64_pipe_issue_pct": 82.7,
                "fp64_pipe_note": ("ncu sm__inst_executed_pipe_fp64 of the largest instance, eri_kernel<2,0,1> "
                                   "(--set full, small case): the stage is FP64-issue bound; the flop "
                                   "fraction is lower because its FP64 instructions mix DMUL/DADD (1 flop) "
                                   "with DFMA (2) while the DGEMM peak issues only DFMAs"),
                "units": (f"executed FP64 flops of the job's eri_kernel launches (ncu instruction "
                          f"counters, DFMA = 2): {flops:.4g}; plus {EXEC_FLOPS[wl][1]:.4g} FP32 FFMA flops "
                          f"of the FP32 tier; {nprim:.4g} primitive quartets before screening")
                if wl in EXEC_FLOPS else f"{nprim:.4g} primitive quartets x FP64 flops per primitive quartet"}

    # the MC stage: HBM-bound.  Algorithmic bytes 32 P S per job (the BF16 hi/lo operands of both
    # sides written once and read once by the tcgen05 GEMM); traffic = the DRAM bytes per sample
    # of the MC kernels from their ncu capture, times the walker pairs
    from slater_stoch_gb300.perfmodel import MC_DRAM_BYTES_PER_SAMPLE
    npair = b.n * (b.n + 1) // 2
    mc_alg = 32.0 * npair * args.walkers
    hbm_peak, hbm_src = 6800.0, "fallback (no MEASURED_PEAKS.json)"
    try:
        hbm_peak = float(json.load(open(Path(__file__).resolve().parent / "MEASURED_PEAKS.json"))["hbm_gbs"])
        hbm_src = "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except (OSError, KeyError, ValueError):
        pass
    mc_ach = mc_alg / t_mc / 1e9
    mc_roofline = {"bound": "hbm", "achieved": mc_ach, "peak": hbm_peak, "unit": "GB/s", "frac": mc_ach / hbm_peak,
                   "peak_source": hbm_src,
                   "traffic": MC_DRAM_BYTES_PER_SAMPLE.get(wl, 0.0) * args.walkers or None,
                   "traffic_note": "DRAM bytes of the MC kernels of one job (ncu capture of one sub-chunk, "
                                   "scaled by the walker pairs)",
                   "kernel": "shared-walker MC stage (sampler, orbital values, operands, tcgen05 GEMM, "
                             "accumulation), timed alone",
                   "units": f"algorithmic bytes 32 P S = {mc_alg:.4g} (P = {npair} function pairs, "
                            f"S = {args.walkers} walker pairs)"}

    if rank == 0:
        lat = sorted(times)
        line = {
            "metric": METRIC,
            "value": value, "unit": "ERIs/s", "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("f64 analytic (f32 for primitive quartets below 1e-11 of their Schwarz bound) + "
                      "bf16x3 (fp32 accumulate) MC"), "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "walkers": args.walkers, "blocks": NBLOCKS, "estimator": "shared-walker, split-BF16",
                       "max_sigma_Ha": max_sigma, "sigma_target_Ha": SIGMA_TARGET,
                       "l2": "flushed (256 MB write) between timed steps", "parallelism": f"replicas x{world}"},
            "p50_ms": lat[len(lat) // 2], "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
            "stages_s": {"analytic": t_analytic, "mc_split_bf16": t_mc},
            "cleanup": cleanup,
            "fp64_plain": {"value": plain_value, "unit": "ERIs/s", "analytic_s": t_analytic,
                           "mc_s_scaled": t_plain_mc, "measured_walkers": plain_npts,
                           "speedup_split_bf16_vs_fp64_plain": value / world / plain_value},
            "e2e": {"value": whole_job_throughput(nint, world, e2e_s), "unit": "ERIs/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "roofline": roofline, "mc_roofline": mc_roofline,
            "clocks": clk.summary(),
            "wall_s_timed": t_wall,
        }
        if world == 1 and not args.no_serving:
            try:
                line["serving"] = serving_run(args.rate, min(args.duration, 10.0), args.large, args.max_running,
                                              max_atoms=args.max_atoms)
            except Exception as ex:  # reported, not fatal for the throughput line
                line["serving"] = {"error": str(ex)}
            try:
                line["batch"] = batch_run(16, 1, 2, max_running=args.max_running)
            except Exception as ex:
                line["batch"] = {"error": str(ex)}
        if world == 1 and not args.no_cpu_baseline:
            cb = cpu_baseline(b, q)
            line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
