"""Asynchronous job API (ss_job_submit / ss_job_poll / ss_job_result) through the C ABI.

Two jobs with different seeds are in flight at once on one context; each must reproduce the
synchronous ss_two_e_job with the same parameters (the job is deterministic for a given seed:
fixed reduction orders everywhere), and the submitting context must stay usable while they run.
"""
import time

import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, configs
from slater_stoch_gb300._lib import SSError

pytestmark = pytest.mark.gpu


def _ctx(b, q):
    ctx = api.Context(0)
    ctx.set_basis(b)
    ctx.set_quartets(*q)
    return ctx


def test_jobs_match_synchronous_job():
    b = configs.h2o_minimal(ng0=6)
    q = basis.build_mapping(b.n)
    args = dict(a_zv=1.8, npts=8192, nblocks=4, estimator="shared", precision="split_bf16")
    with _ctx(b, q) as ctx:
        ids = [ctx.job_submit(seed=s, **args) for s in (3, 4)]
        g, _ = ctx.gauss_eri()  # the submitting context keeps working meanwhile
        t0 = time.time()
        while not all(ctx.job_poll(i) for i in ids):
            assert time.time() - t0 < 120
            time.sleep(0.01)
        res = [ctx.job_result(i) for i in ids]
        ref = [ctx.two_e_job(seed=s, **args) for s in (3, 4)]
    for (e, s), (er, sr) in zip(res, ref):
        np.testing.assert_allclose(e, er, rtol=1e-14, atol=1e-17)
        np.testing.assert_allclose(s, sr, rtol=1e-12, atol=1e-17)
    assert not np.array_equal(res[0][0], res[1][0])  # the seeds differ
    assert np.max(np.abs(res[0][0] - g)) < 1e-2  # analytic + a small correction


def test_job_errors_are_reported():
    b = configs.h2o_minimal(ng0=4)
    q = basis.build_mapping(b.n)
    with _ctx(b, q) as ctx:
        jid = ctx.job_submit(1.8, 1, 8192, 2, "shared", "fp64")  # shared runs split-BF16 only
        with pytest.raises(SSError, match="SPLIT_BF16"):
            ctx.job_result(jid)
        with pytest.raises(SSError, match="unknown job"):
            ctx.job_poll(jid)


def test_job_admission_limits():
    """Jobs admitted one at a time (max_running = 1) reproduce the synchronous job and never
    overlap; a job whose ERI-buffer footprint exceeds the budget is refused at submission."""
    b = configs.h2o_minimal(ng0=6)
    q = basis.build_mapping(b.n)
    args = dict(a_zv=1.8, npts=8192, nblocks=2, estimator="shared", precision="split_bf16")
    with _ctx(b, q) as ctx:
        foot = ctx.job_footprint()
        assert foot == 96 * len(q[0])
        ctx.job_limits(max_running=1)
        ids = [ctx.job_submit(seed=s, **args) for s in (3, 4, 5)]
        res = [ctx.job_result(i) for i in ids]
        st = ctx.job_stats()
        assert st["peak_running"] == 1 and st["running"] == 0 and st["queued"] == 0
        assert st["peak_bytes"] == foot
        ref = ctx.two_e_job(seed=5, **args)
        np.testing.assert_allclose(res[2][0], ref[0], rtol=1e-14, atol=1e-17)
        ctx.job_limits(eri_budget_bytes=foot // 2)
        with pytest.raises(SSError, match="budget"):
            ctx.job_submit(seed=6, **args)


@pytest.mark.parametrize("estimator,precision", [("shared", "split_bf16"), ("faithful", "fp64")])
def test_two_e_job_matches_staged_calls(estimator, precision):
    """ss_two_e_job runs the analytic stage on its own stream beside the MC; the result is bitwise
    that of the staged calls ss_gauss_eri, ss_zvmc and ss_combine on one stream, and the
    context's later calls see the finished analytic stage."""
    b = configs.h2o_26(ng0=6)
    q = basis.build_mapping(b.n)
    npts = 8000 if estimator == "faithful" else 1 << 16
    with _ctx(b, q) as ctx:
        e_job, s_job = ctx.two_e_job(1.8, 7, npts, 3, estimator, precision)
        g_after, _ = ctx.gauss_eri()
        ctx.invalidate()
        g, _ = ctx.gauss_eri()
        m, s = ctx.zvmc(1.8, 7, npts, 3, estimator, precision)
        e = ctx.combine()
    assert np.array_equal(g_after, g)
    assert np.array_equal(e_job, e)
    assert np.array_equal(s_job, s)
