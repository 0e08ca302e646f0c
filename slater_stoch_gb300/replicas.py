"""Replica bookkeeping for runs on N GPUs of one node (one process per GPU).

The two-electron job does not need a collective on its data path at the sizes run here: each
rank runs whole jobs of its own (its own Philox seed), so N ranks process N jobs.  The reference's
MPI split (walker streams per rank plus one Allreduce of the per-quartet sums,
src/two_e_slater.F90:499-513) is the exchange a sharded single job would need; with one GPU per
box it is not built.  What the ranks share is the clock: every timed region is bracketed by a
barrier and the slowest rank's time is the job time.
"""
from __future__ import annotations


def job_seed(base_seed: int, rank: int) -> int:
    """Philox seed of the rank's jobs (independent walker streams per rank)."""
    return int(base_seed) + int(rank)


def max_over_ranks(x: float, world: int, dist=None, device="cpu") -> float:
    """The maximum of a per-rank float over all ranks (all_reduce MAX; identity for one rank)."""
    if world <= 1 or dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_throughput(nint: int, world: int, seconds_per_job: float) -> float:
    """Unique ERIs per second of all ranks together: each rank finishes one job of nint ERIs per
    step, the step lasting as long as the slowest rank's."""
    return world * nint / seconds_per_job
