"""GPU ZV-MC estimators vs the CPU oracle on identical samples.

Faithful estimator (src/two_e_slater.F90:386-496): the GPU draws Philox walkers, the same
walkers are copied to the host and fed to the oracle.  Gate: the plain FP64 path matches per
integral to 1e-10 relative, |dmean| <= 1e-10 |ERI| + 1e-14 S_q, with ERI the analytic value plus
the correction and S_q = sqrt((ik|ik)(jl|jl)) the Schwarz bound (the magnitude of the separately
accumulated STO and fit sums, whose FP64 rounding limits a correction that is their difference);
the block error bar to |dsigma| <= 1e-6 sigma + 1e-14 S_q.

Shared estimator, split-BF16 tensor-core contraction: the oracle evaluates the same
estimator in FP64 on the same samples (u1, u2, w).  Gate: per integral
|gpu - fp64| <= 0.1 sigma_MC and <= 1e-8 Ha.
"""
import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, configs

pytestmark = pytest.mark.gpu


def _setup(cfg, ng0):
    b = getattr(configs, cfg)(ng0=ng0)
    q = basis.build_mapping(b.n)
    return b, q


_PRE = {}


def _oracle_precond(O, ob, key):
    if key not in _PRE:
        O.set_sum_mode("extended")
        _PRE[key] = O.precond(ob)
    return _PRE[key]


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-10), ("ref32", 1e-9)])
@pytest.mark.parametrize("cfg,ng0", [("h2o_minimal", 4), ("h2o_minimal", 20), ("h2o_26", 20)])
def test_faithful_vs_oracle(cfg, ng0, precision, rtol):
    """h2o_26 with 20-Gaussian fits is the benchmarked workload (61,776 quartets); there the
    |ERI| in the gate's relative term is the device's analytic value, which the analytic parity
    tests hold to 1e-12 of the oracle."""
    from oracle import binding as O
    b, q = _setup(cfg, ng0)
    nblocks, npts = 3, 4000
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        mean, sigma = ctx.zvmc(a_zv=1.8, seed=7, npts=npts, nblocks=nblocks, precision=precision)
        r1, r2 = ctx.draw_walkers(seed=7, first=0, S=nblocks * npts)
        # same walkers through the host-walker entry point
        mean_w, sigma_w = ctx.zvmc_walkers(1.8, r1, r2, npts, nblocks, precision)
        g_dev, _ = ctx.gauss_eri() if cfg == "h2o_26" else (None, 0)
    ob = O.OracleBasis(b)
    ref, err = O.zvmc_faithful(ob, q, 1.8, r1, r2, nblocks, npts, precision)
    pre = _oracle_precond(O, ob, (cfg, ng0)).reshape(b.n, b.n, order="F")
    gauss = g_dev if g_dev is not None else O.gauss_eri(ob, q, pre.reshape(-1, order="F"))[0]
    i, j, k, l = [np.asarray(a) - 1 for a in q]
    schwarz = np.sqrt(np.abs(pre[i, k] * pre[j, l]))
    bound = rtol * np.abs(gauss + ref) + 1e-14 * schwarz
    d = np.abs(mean - ref)
    assert np.all(d <= bound), np.max(d / bound)
    # sigma: the block means carry the same FP64 summation noise as the means (1e-14 S_q)
    assert np.all(np.abs(sigma - err) <= 1e-6 * err + 1e-14 * schwarz)
    np.testing.assert_array_equal(mean, mean_w)


def test_walkers_are_standard_normal():
    b, q = _setup("h2o_minimal", 4)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        r1, r2 = ctx.draw_walkers(seed=1, first=0, S=200000)
        a1, _ = ctx.draw_walkers(seed=1, first=1000, S=10)
    x = np.concatenate([r1.ravel(), r2.ravel()])
    assert abs(x.mean()) < 5e-3 and abs(x.std() - 1) < 5e-3
    np.testing.assert_array_equal(a1, r1[1000:1010])  # counter-based: any range regenerates


@pytest.mark.parametrize("cfg,ng0,npts,nblocks", [("h2o_minimal", 4, 8192, 4), ("h2o_26", 20, 4096, 3)])
def test_shared_split_bf16_vs_fp64(cfg, ng0, npts, nblocks):
    from oracle import binding as O
    b, q = _setup(cfg, ng0)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        mean, sigma = ctx.zvmc(a_zv=1.8, seed=11, npts=npts, nblocks=nblocks, estimator="shared",
                               precision="split_bf16")
        u1, u2, w = ctx.shared_samples(1.8, seed=11, first=0, S=nblocks * npts)
    ob = O.OracleBasis(b)
    ref, err = O.zvmc_shared(ob, q, u1, u2, w, nblocks, npts, symmetrize=True)
    d = np.abs(mean - ref)
    assert np.all(d <= 0.1 * err + 1e-15), f"max |d|/sigma {np.max(d / np.maximum(err, 1e-300)):.3g}"
    if ng0 == 20:  # the absolute gate is stated for the production 20-Gaussian fits, whose
        assert d.max() <= 1e-8, d.max()  # corrections are ~1e-7 Ha (4-Gaussian ones are ~1e-2 Ha)
    np.testing.assert_allclose(sigma, err, rtol=0.05, atol=1e-12)


@pytest.mark.parametrize("zeta", [1.0, 1.7])
def test_shared_estimator_sto_1s_known_answer(zeta):
    """Analytic fit ERI + shared-walker correction = the exact unnormalised 1s STO
    self-repulsion 5 pi^2 / (8 zeta^5) within 4 sigma (3-Gaussian fit: the fit alone is off by
    many sigma), so the sampler's mixture density and weights carry no bias."""
    import math
    mol = basis.molecule_bohr(["H"], [[0.0, 0.0, 0.0]])
    b = basis.build_basis(mol, {1: [("1S", zeta)]}, basis.FitParams(ng0=3))
    q = basis.build_mapping(1)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        eri, sig = ctx.two_e_job(1.8, 7, 1 << 17, 10, "shared", "split_bf16")
        g, _ = ctx.gauss_eri()
    exact = 5 * math.pi ** 2 / (8 * zeta ** 5)
    assert abs(g[0] - exact) > 10 * sig[0]
    assert abs(eri[0] - exact) <= 4 * sig[0], (eri[0], exact, sig[0])


def test_shared_agrees_with_faithful():
    """Both estimators are unbiased for the same correction: on the 7-function H2O basis with
    4-Gaussian fits (corrections ~1e-2 Ha), two independent runs (different seeds, different
    estimators) agree within 3 combined sigma.  With 406 integrals and |z| ~ N(0,1), about
    406 * 0.0027 = 1.1 exceed 3 sigma; the gate allows at most 6 exceedances (the chance of
    more is ~1e-4 for independent integrals), none beyond 5 sigma, and mean |z| < 1.2 (|N(0,1)|
    averages 0.80)."""
    b, q = _setup("h2o_minimal", 4)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        ms, ss = ctx.zvmc(a_zv=1.8, seed=21, npts=1 << 16, nblocks=16, estimator="shared",
                          precision="split_bf16")
        mf, sf = ctx.zvmc(a_zv=1.8, seed=22, npts=40 * 400, nblocks=16, estimator="faithful",
                          precision="fp64")
    z = np.abs(ms - mf) / np.sqrt(ss ** 2 + sf ** 2 + 1e-300)
    n3 = int((z > 3.0).sum())
    assert n3 <= 6, f"{n3} of {z.size} integrals beyond 3 sigma (expected ~1.1), max |z| {z.max():.2f}"
    assert np.all(z <= 5.0), f"max |z| {z.max():.2f}"
    assert np.mean(z) < 1.2
