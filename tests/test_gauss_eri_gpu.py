"""GPU analytic Gaussian-fit ERIs vs the CPU oracle (restated gauss_ijkl, src/gauss_ijkl.F90).

Tolerance (analytic Gaussian ERIs to 1e-12): per integral
|gpu - oracle| <= 1e-12 * |oracle| + 1e-12 * sqrt(precond_ik * precond_jl),
the second term covers integrals that vanish by symmetry (both sides are ~1e-20).
"""
import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, configs

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _oracle():
    """Oracle with the exactly-summed accumulation: the reference's own sequential FP64 sum over
    up to ~1e7 primitive terms carries ~1e-12 relative rounding (test_oracle_summation_error)."""
    from oracle import binding as O
    O.set_sum_mode("extended")
    return O


def _check(g, ref, pre, q):
    n = int(round(np.sqrt(pre.size)))
    P = pre.reshape(n, n, order="F")
    i, j, k, l = [np.asarray(a) - 1 for a in q]
    scale = np.sqrt(np.abs(P[i, k] * P[j, l]))
    err = np.abs(g - ref)
    bound = RTOL * np.abs(ref) + RTOL * scale
    bad = np.nonzero(err > bound)[0]
    assert bad.size == 0, (f"{bad.size} quartets outside tolerance; worst rel "
                           f"{(err / np.maximum(np.abs(ref), 1e-300))[bad].max():.3e}")


@pytest.mark.parametrize("cfg,ng0", [("h2o_minimal", 4), ("h2o_minimal", 6), ("h2o_26", 3)])
def test_gauss_eri_full_small_fits(cfg, ng0):
    O = _oracle()
    b = getattr(configs, cfg)(ng0=ng0)
    q = basis.build_mapping(b.n)
    ob = O.OracleBasis(b)
    pre = O.precond(ob)
    ref, nz_ref = O.gauss_eri(ob, q, pre)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        gp = ctx.precond()
        g, nz = ctx.gauss_eri()
    np.testing.assert_allclose(gp.reshape(-1, order="F"), pre, rtol=RTOL, atol=0)
    assert nz == nz_ref
    _check(g, ref, pre, q)


def test_gauss_eri_golden_ng20():
    """20-Gaussian fits (the production setting) against the committed oracle fixture."""
    from pathlib import Path
    fx = np.load(Path(__file__).parent / "golden" / "gauss_eri_h2o_minimal_ng20.npz")
    b = configs.h2o_minimal(ng0=20)
    q = basis.build_mapping(b.n)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        g, nz = ctx.gauss_eri()
    _check(g, fx["eri_ext"], fx["precond"], q)
