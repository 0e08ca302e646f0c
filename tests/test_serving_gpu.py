"""The serving loop (slater_stoch_gb300/serving.py) on the GPU: open-loop Poisson arrivals of
jobs of uneven size with per-job error-bar targets, run concurrently through the job API, each
retired at its target.  Every result must equal the same request run alone on a fresh context
(the jobs are deterministic for their seed: fixed reduction orders everywhere), to the
tolerance of the job API's own test: 1e-14 relative on the ERIs, 1e-12 on the error bars."""
import numpy as np
import pytest

from slater_stoch_gb300 import serving

pytestmark = pytest.mark.gpu


def test_results_in_the_mix_equal_results_alone():
    reqs = serving.make_requests(seed=7, rate_per_s=400.0, duration_s=0.05, large_fraction=0.2,
                                 sigma_range=(1e-6, 1e-4))
    assert len(reqs) >= 8
    rep = serving.serve(reqs, max_running=4, npts=1 << 14, nblocks_max=16, keep_results=True)
    s = rep.summary()
    assert s["jobs"] == len(reqs) and len(rep.results) == len(reqs)
    assert s["peak_running"] >= 2  # jobs overlapped on the device
    assert s["p99_ms"] >= s["p50_ms"] > 0
    # a job stops early only at its target: a job that used fewer blocks than allowed reached it
    for b, r in zip(rep.blocks, sorted(reqs, key=lambda x: x.arrival_s)):
        assert 2 <= b <= 16
    assert s["jobs_at_sigma_target"] >= 1
    picks = [r for r in reqs if r.label == "large"][:1] + [r for r in reqs if r.label == "small"][:3]
    for r in picks:
        eri, sig = serving.run_alone(r, npts=1 << 14, nblocks_max=16)
        e_mix, s_mix = rep.results[r.rid]
        np.testing.assert_allclose(e_mix, eri, rtol=1e-14, atol=1e-17)
        np.testing.assert_allclose(s_mix, sig, rtol=1e-12, atol=1e-17)


def test_admission_budget_limits_concurrency():
    """With an ERI budget that holds only one of the large jobs, no two of them run together
    (small ones may run beside them), and every job still completes."""
    from slater_stoch_gb300 import basis, configs
    from slater_stoch_gb300._lib import load
    big = configs.h2o_minimal(ng0=6)
    foot = int(load().ss_job_footprint(len(basis.build_mapping(big.n)[0])))
    reqs = serving.make_requests(seed=3, rate_per_s=500.0, duration_s=0.02, large_fraction=1.0,
                                 large=big, sigma_range=(1e-4, 1e-3), ng0=6)
    rep = serving.serve(reqs, eri_budget_bytes=foot, max_running=8, npts=1 << 13, nblocks_max=4)
    assert rep.summary()["jobs"] == len(reqs) and rep.peak_running == 1
