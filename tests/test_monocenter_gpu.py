"""Exact one-centre Slater ERIs on the device (the do_exact_monocenter path of
src/two_e_slater.F90:318-369) against the oracle's restatement of compute_int_slater, and their
use in the merged ERIs."""
import numpy as np
import pytest

from oracle import binding as O
from slater_stoch_gb300 import api, basis, configs

pytestmark = pytest.mark.gpu


def _ctx(b, q):
    ctx = api.Context(0)
    ctx.set_basis(b)
    ctx.set_quartets(*q)
    return ctx


def test_monocenter_matches_oracle():
    """Every quartet of the 26-function list: same one-centre mask (9,556 quartets), values to
    1e-13 relative (same closed forms; rounding differs by contraction only)."""
    b = configs.h2o_26(ng0=20)
    q = basis.build_mapping(b.n)
    ref, rmask = O.monocenter(O.OracleBasis(b), q)
    with _ctx(b, q) as ctx:
        got, mask = ctx.monocenter()
    assert np.array_equal(mask, rmask) and mask.sum() == 9556
    assert np.all(got[~mask] == 0.0)
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-13


def test_monocenter_agrees_with_gaussian_fits():
    """The 20-Gaussian-fit ERIs of all one-centre quartets reproduce the exact Slater values to
    1e-6 relative (or 1e-10 absolute for the near-zero ones)."""
    b = configs.h2o_26(ng0=20)
    q = basis.build_mapping(b.n)
    with _ctx(b, q) as ctx:
        ex, mask = ctx.monocenter()
        g, _ = ctx.gauss_eri()
    d = np.abs(g[mask] - ex[mask])
    assert np.all(d <= 1e-6 * np.abs(ex[mask]) + 1e-10), d.max()


def test_exact_monocenter_in_job():
    """With the exact one-centre path on, the merged ERI of a one-centre quartet is its exact
    value with error bar 0; every other quartet is bit-identical to the run without it."""
    b = configs.h2o_minimal(ng0=20)
    q = basis.build_mapping(b.n)
    with _ctx(b, q) as ctx:
        e0, s0 = ctx.two_e_job(a_zv=1.8, seed=3, npts=1 << 14, nblocks=4)
        ex, mask = ctx.monocenter()
        ctx.set_exact_monocenter(True)
        e1, s1 = ctx.two_e_job(a_zv=1.8, seed=3, npts=1 << 14, nblocks=4)
        jid = ctx.job_submit(a_zv=1.8, seed=3, npts=1 << 14, nblocks=4)
        e2, s2 = ctx.job_result(jid)
    assert mask.sum() > 0
    assert np.array_equal(e1[mask], ex[mask]) and np.all(s1[mask] == 0.0)
    assert np.array_equal(e1[~mask], e0[~mask]) and np.array_equal(s1[~mask], s0[~mask])
    assert np.array_equal(e2, e1) and np.array_equal(s2, s1)
    # the MC-corrected fit values scatter around the exact ones within their error bars
    ok = mask & (s0 > 0)
    z = np.abs(e0[ok] - ex[ok]) / s0[ok]
    assert ok.sum() > 0 and np.median(z) < 2.0
