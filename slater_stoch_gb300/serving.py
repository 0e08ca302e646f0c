"""Continuous-batching request loop over the asynchronous job API (the serving workload).

The reference runs one integral job per process (src/two_e_slater.F90:219-564); a service
receives jobs as they arrive.  Here requests arrive open loop -- a seeded Poisson process, each
request carrying its own system, seed and error-bar target -- and every request is submitted the
moment it arrives (``ss_job_submit_inputs``), whatever is still running.  The library admits the
queued jobs in arrival order as running jobs finish and free their slots and ERI-buffer
footprint (``ss_job_limits``), runs the admitted ones concurrently on pooled worker contexts
(their own CUDA streams), and retires each at the first MC block boundary where its largest
error bar is at or below its target (the reference's error_max, src/two_e_slater.F90:538-553).
Latency is completion minus arrival; throughput is unique ERIs completed per second.

Every job is deterministic for its seed (fixed reduction orders on the device), so a request's
result is the same whether it ran alone or in the mix (``tests/test_serving_gpu.py``).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import api, basis, configs


@dataclass
class Request:
    rid: int
    arrival_s: float           # seconds after the start of the run
    basis: object              # basis.Basis of the request's system
    quartets: tuple            # 1-based (is, js, ks, ls) of its unique quartets
    sigma_target: float        # Ha
    seed: int
    label: str = ""

    @property
    def nint(self) -> int:
        return len(self.quartets[0])


def small_system(rng: np.random.Generator, ng0: int = 20, max_atoms: int = 2):
    """A system drawn with the random-molecule rules (Z in {1,6,7,8}; heavy atoms 1s 2s 2p 3d,
    H 1s 2p; Slater-rule exponents x U[0.8, 1.2]) with 1..max_atoms atoms in a 4-bohr box."""
    na = int(rng.integers(1, max_atoms + 1))
    return configs.random_molecule(int(rng.integers(0, 2 ** 31 - 1)), natoms=na, box=4.0, min_sep=2.0, ng0=ng0)


def make_requests(seed: int, rate_per_s: float, duration_s: float, large_fraction: float = 0.05,
                  sigma_range=(1e-7, 1e-5), max_atoms: int = 2, large=None, ng0: int = 20) -> list[Request]:
    """Seeded open-loop arrivals: exponential inter-arrival times of mean 1/rate over
    duration_s; each request is a small random system, or with probability large_fraction the
    `large` system (default: the 7-function H2O); sigma targets log-uniform in sigma_range."""
    rng = np.random.default_rng(seed)
    big = large if large is not None else configs.h2o_minimal(ng0=ng0)
    big_q = basis.build_mapping(big.n)
    out, t, rid = [], 0.0, 0
    lo, hi = math.log(sigma_range[0]), math.log(sigma_range[1])
    while True:
        t += float(rng.exponential(1.0 / rate_per_s))
        if t > duration_s:
            break
        if rng.random() < large_fraction:
            b, q, label = big, big_q, "large"
        else:
            b = small_system(rng, ng0=ng0, max_atoms=max_atoms)
            q, label = basis.build_mapping(b.n), "small"
        out.append(Request(rid, t, b, tuple(q), float(math.exp(rng.uniform(lo, hi))),
                           int(rng.integers(1, 2 ** 31 - 1)), label))
        rid += 1
    return out


@dataclass
class ServeReport:
    n_jobs: int
    wall_s: float
    eris: int
    latency_s: list = field(default_factory=list)
    run_s: list = field(default_factory=list)
    wait_s: list = field(default_factory=list)
    blocks: list = field(default_factory=list)
    sigma_ok: int = 0
    peak_running: int = 0
    peak_bytes: int = 0
    results: dict = field(default_factory=dict)

    def summary(self) -> dict:
        lat = np.sort(np.asarray(self.latency_s))
        pct = lambda p: float(lat[min(len(lat) - 1, int(math.ceil(p * len(lat))) - 1)]) if len(lat) else None
        return {"jobs": self.n_jobs, "wall_s": self.wall_s, "unique_eris": self.eris,
                "eris_per_s": self.eris / self.wall_s if self.wall_s > 0 else None,
                "p50_ms": 1e3 * pct(0.50) if len(lat) else None, "p99_ms": 1e3 * pct(0.99) if len(lat) else None,
                "mean_run_ms": 1e3 * float(np.mean(self.run_s)) if self.run_s else None,
                "mean_wait_ms": 1e3 * float(np.mean(self.wait_s)) if self.wait_s else None,
                "jobs_at_sigma_target": self.sigma_ok, "mean_blocks": float(np.mean(self.blocks)) if self.blocks else None,
                "peak_running": self.peak_running, "peak_eri_bytes": self.peak_bytes}


def serve(requests: list[Request], device: int = 0, eri_budget_bytes: int = 150 * 10 ** 9,
          max_running: int = 8, a_zv: float = 1.8, npts: int = 1 << 16, nblocks_max: int = 64,
          keep_results: bool = False, poll_s: float = 0.0002) -> ServeReport:
    """Run the requests open loop on one GPU; returns latencies and throughput."""
    reqs = sorted(requests, key=lambda r: r.arrival_s)
    done_at: dict[int, float] = {}
    rep = ServeReport(n_jobs=len(reqs), wall_s=0.0, eris=0)
    with api.Context(device) as ctx:
        ctx.job_limits(eri_budget_bytes, max_running)
        inflight: dict[int, Request] = {}
        nxt = 0
        t0 = time.perf_counter()
        while nxt < len(reqs) or inflight:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and reqs[nxt].arrival_s <= now:  # open loop: submit on arrival
                r = reqs[nxt]
                jid = ctx.job_submit_inputs(r.basis, r.quartets, a_zv, r.seed, npts, nblocks_max, "shared",
                                            "split_bf16", r.sigma_target)
                inflight[jid] = r
                nxt += 1
            for jid in [j for j in inflight if ctx.job_poll(j)]:
                t_done = time.perf_counter() - t0
                r = inflight.pop(jid)
                info = ctx.job_info(jid)
                eri, sig = ctx.job_result(jid)
                done_at[r.rid] = t_done
                rep.latency_s.append(t_done - r.arrival_s)
                rep.run_s.append(info["run_s"])
                rep.wait_s.append(info["wait_s"])
                rep.blocks.append(info["blocks"])
                rep.sigma_ok += int(info["max_sigma"] <= r.sigma_target)
                rep.eris += r.nint
                if keep_results:
                    rep.results[r.rid] = (eri, sig)
            if nxt < len(reqs) and not inflight:
                time.sleep(max(0.0, min(reqs[nxt].arrival_s - (time.perf_counter() - t0), 0.01)))
            else:
                time.sleep(poll_s)
        rep.wall_s = (max(done_at.values()) if done_at else 0.0)
        st = ctx.job_stats()
        rep.peak_running, rep.peak_bytes = st["peak_running"], st["peak_bytes"]
    return rep


def run_alone(r: Request, device: int = 0, a_zv: float = 1.8, npts: int = 1 << 16, nblocks_max: int = 64):
    """The same request as a synchronous job on a fresh context (the reference for the mix)."""
    with api.Context(device) as ctx:
        ctx.set_basis(r.basis)
        ctx.set_quartets(*r.quartets)
        return ctx.two_e_job(a_zv, r.seed, npts, nblocks_max, "shared", "split_bf16", r.sigma_target)
