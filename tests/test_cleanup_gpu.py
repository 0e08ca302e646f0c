"""PSD cleanup (svd_clean, davidson_clean's exact projection) and Davidson on the GPU vs the
numpy oracle.

Inputs: analytic ERIs plus a seeded symmetric perturbation sized to give the ERI matrix
negative eigenvalues (as MC noise does).  Both sides draw the same Philox test matrices.

* svd_clean: where one pass covers the whole matrix (rank = N) the GPU matches the reference
  algorithm to 1e-9 of the largest ERI.  With rank < N the reference's sign test is a knife
  edge for components whose +/- partners are nearly degenerate (they are noise-level), so the
  two agree to the perturbation's size; both reduce the negative part.
* exact projection: matches the oracle to 1e-12 of the largest ERI, and with the packed
  Coulomb metric the cleaned matrix is PSD to -1e-12 (the PSD gate of the cleanup).
* Davidson: lowest 10 eigenvalues against numpy.linalg.eigh to 1e-8 of the spectrum.
"""
import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, configs

pytestmark = pytest.mark.gpu


def _noisy_eris(cfg, ng0, layout, seed=5):
    from oracle import cleanup as OC
    b = getattr(configs, cfg)(ng0=ng0)
    q = basis.build_mapping(b.n)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        g, _ = ctx.gauss_eri()
    return b, q, g, OC.perturb_indefinite(g, q, b.n, layout, seed=seed)


@pytest.mark.parametrize("cfg,layout,rank,over,qq", [("h2o_minimal", "packed_pair", 28, 0, 4),
                                                      ("h2o_minimal", "ref_n2", 49, 0, 12),
                                                      ("h2o_26", "packed_pair", 200, 10, 4)])
def test_svd_clean_matches_oracle(cfg, layout, rank, over, qq):
    from oracle import cleanup as OC
    b, q, g, moy = _noisy_eris(cfg, 6, layout)
    lmin0 = np.linalg.eigvalsh(OC.matrix_from_eris(moy, q, b.n, layout)).min()
    assert lmin0 < -1e-8  # the perturbation made it indefinite
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        got, nrem = ctx.psd_clean(moy, layout=layout, rank=rank, oversample=over, q=qq, seed=3)
    ref, nrem_ref = OC.svd_clean(moy, q, b.n, layout, rank, over, qq, seed=3)
    lmin = np.linalg.eigvalsh(OC.matrix_from_eris(got, q, b.n, layout)).min()
    assert nrem > 0 and lmin > lmin0
    scale = np.abs(moy).max()
    pert = np.abs(moy - g).max()
    full_rank = min(rank + over, len(OC.matrix_from_eris(moy, q, b.n, layout))) == len(
        OC.matrix_from_eris(moy, q, b.n, layout))
    tol = 1e-9 * scale if full_rank else 10 * pert
    assert np.max(np.abs(got - ref)) <= tol, np.max(np.abs(got - ref))


@pytest.mark.parametrize("cfg,layout", [("h2o_minimal", "packed_pair"), ("h2o_26", "packed_pair"),
                                        ("h2o_minimal", "ref_n2")])
def test_psd_project_exact(cfg, layout):
    from oracle import cleanup as OC
    b, q, g, moy = _noisy_eris(cfg, 6, layout)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        got, nrem = ctx.psd_project(moy, layout=layout)
    ref, nrem_ref = OC.psd_project(moy, q, b.n, layout)
    assert nrem == nrem_ref and nrem > 0
    scale = np.abs(moy).max()
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale * 10
    if layout == "packed_pair":
        assert np.linalg.eigvalsh(OC.matrix_from_eris(got, q, b.n, layout)).min() >= -1e-12


def test_psd_project_rank_deficient_metric():
    """The exact analytic Coulomb metric of the H2O 26-function basis is PSD with a numerical
    null space (eigenvalues at rounding level, ~1e-16 of the largest); its tridiagonal form
    carries a long run of rounding-level entries that the eigensolver must deflate."""
    from oracle import cleanup as OC
    b = configs.h2o_26(ng0=6)
    q = basis.build_mapping(b.n)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        g, _ = ctx.gauss_eri()
        got, nrem = ctx.psd_project(g, layout="packed_pair")
    ev = np.linalg.eigvalsh(OC.matrix_from_eris(g, q, b.n, "packed_pair"))
    assert ev.min() > -1e-13 * ev.max()  # the input is PSD to rounding
    # only rounding-level components are removed (their signs are noise, so their count is not
    # compared with numpy's)
    assert 0 <= nrem < len(ev)
    assert np.max(np.abs(got - g)) <= 1e-13 * np.abs(g).max()


def test_clean_pipeline_is_psd():
    """svd_clean with the 26-function workload's parameters (rank 200, oversampling 10, 4 power
    iterations on the 351x351 packed metric) followed by the exact projection: PSD to -1e-12."""
    from oracle import cleanup as OC
    b, q, g, moy = _noisy_eris("h2o_26", 6, "packed_pair")
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        c1, _ = ctx.psd_clean(moy, layout="packed_pair", rank=200, oversample=10, q=4, seed=3)
        c2, _ = ctx.psd_project(c1, layout="packed_pair")
    assert np.linalg.eigvalsh(OC.matrix_from_eris(c2, q, b.n, "packed_pair")).min() >= -1e-12
    assert np.max(np.abs(c2 - moy)) <= 10 * np.abs(moy - g).max()


def test_davidson_lowest_eigenpairs():
    """Lowest 10 eigenpairs of the cleaned packed metric (whose low end is a cluster of
    near-zero eigenvalues; the reference's correction-norm criterion 1e-8 needs thousands of
    iterations there, 1e-6 pins the eigenvalues to ~1e-10)."""
    from oracle import cleanup as OC
    b, q, g, noisy = _noisy_eris("h2o_26", 6, "packed_pair")
    moy, _ = OC.psd_project(noisy, q, b.n, "packed_pair")
    H = OC.matrix_from_eris(moy, q, b.n, "packed_pair")
    full = np.linalg.eigvalsh(H)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        ev, vec = ctx.davidson(moy, m=10, layout="packed_pair", tol=1e-6, max_iter=3000)
    spread = np.abs(full).max()
    assert np.max(np.abs(np.sort(ev) - full[:10])) <= 1e-8 * spread
    res = H @ vec - vec * ev[None, :]
    assert np.max(np.linalg.norm(res, axis=0)) < 1e-5 * spread


@pytest.mark.parametrize("cfg,block,blocks", [("h2o_minimal", 7, 4), ("h2o_26", 27, 13)])
def test_davidson_clean_matches_exact_projection(cfg, block, blocks):
    """Matrix-free Davidson cleanup (davidson_clean's nbasis >= 200 path) on the packed metric
    with a basis that can grow to the whole space (block x blocks = N): only converged
    negative eigenpairs are deflated and the packed canonical read-back is exact, so the
    result is the exact projection's to 1e-11 of the largest ERI."""
    from oracle import cleanup as OC
    b, q, g, moy = _noisy_eris(cfg, 6, "packed_pair")
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        got, nrem = ctx.davidson_clean(moy, layout="packed_pair", block=block, max_blocks=blocks, tol=1e-8)
    ref, nref = OC.psd_project(moy, q, b.n, "packed_pair")
    scale = np.abs(moy).max()
    diff = np.max(np.abs(got - ref)) / scale
    lmin = np.linalg.eigvalsh(OC.matrix_from_eris(got, q, b.n, "packed_pair")).min()
    # a converged Ritz pair (residual < tol) leaves a rounding-level remainder that a later
    # search may deflate as well, so the count can exceed the exact projection's
    assert nrem >= nref > 0 and diff <= 1e-11 and lmin >= -1e-11, (nrem, nref, diff, lmin)


def test_davidson_clean_restarted_basis():
    """The reference's default block and basis size (nbasis = 26 vectors, 26 blocks, capped at
    338 of the 351 dimensions) restart the search; the deflations still reach the exact
    projection to 1e-9 of the largest ERI and leave no eigenvalue below -1e-10."""
    from oracle import cleanup as OC
    b, q, g, moy = _noisy_eris("h2o_26", 6, "packed_pair")
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        got, nrem = ctx.davidson_clean(moy, layout="packed_pair", tol=1e-8, max_iter=5000)
    ref, _ = OC.psd_project(moy, q, b.n, "packed_pair")
    assert nrem > 0
    assert np.max(np.abs(got - ref)) <= 1e-9 * np.abs(moy).max()
    assert np.linalg.eigvalsh(OC.matrix_from_eris(got, q, b.n, "packed_pair")).min() >= -1e-10


def test_davidson_clean_ref_n2_fixed_point():
    """REF_N2 (the reference's n^2 x n^2 <ij|kl> matrix): the canonical read-back of a rank-one
    deflation does not keep the matrix's 8-fold index symmetry, so searches and deflations
    repeat until the rebuilt matrix has no eigenvalue below rounding level (-1e-12); the
    change stays of the size of the perturbation."""
    from oracle import cleanup as OC
    b, q, g, moy = _noisy_eris("h2o_minimal", 6, "ref_n2")
    lmin0 = np.linalg.eigvalsh(OC.matrix_from_eris(moy, q, b.n, "ref_n2")).min()
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        got, nrem = ctx.davidson_clean(moy, layout="ref_n2", tol=1e-8, max_iter=5000)
    assert lmin0 < -1e-8 and nrem > 0
    assert np.linalg.eigvalsh(OC.matrix_from_eris(got, q, b.n, "ref_n2")).min() >= -1e-12
    assert np.max(np.abs(got - moy)) <= 10 * np.abs(moy - g).max()
