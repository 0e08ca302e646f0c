"""Edge cases of the analytic ERIs through the C ABI: a one-function basis (its only quartet is
the Schwarz diagonal), an empty quartet list, a malformed quartet, and quartet lists given in
another order, with duplicates, or as a subset (each value depends only on its own quartet: equal
to the full canonical list's to 1e-13 relative, the bra-slice split of a quartet depending on
how many quartets share its kernel class)."""
import math

import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, configs
from slater_stoch_gb300._lib import SSError

pytestmark = pytest.mark.gpu


def test_one_function_basis():
    from oracle import binding as O
    O.set_sum_mode("extended")
    mol = basis.molecule_bohr(["H"], [[0.0, 0.0, 0.0]])
    b = basis.build_basis(mol, {1: [("1S", 1.3)]}, basis.FitParams(ng0=20))
    q = basis.build_mapping(1)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        g, _ = ctx.gauss_eri()
    ref = O.gauss_list(O.OracleBasis(b), q)
    assert abs(g[0] - ref[0]) <= 1e-12 * abs(ref[0])
    # the 20-Gaussian fit reproduces the STO 1s self-repulsion 5 pi^2 / (8 zeta^5) (the oracle
    # to 1.6e-12 relative)
    assert abs(g[0] - 5 * math.pi ** 2 / (8 * 1.3 ** 5)) < 1e-10 * g[0]


def test_empty_and_malformed_quartet_lists():
    b = configs.h2o_minimal(ng0=3)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*[np.zeros(0, np.int32)] * 4)
        with pytest.raises(SSError, match="no quartets"):
            ctx.gauss_eri()
        bad = [np.array([1], np.int32), np.array([1], np.int32), np.array([2], np.int32), np.array([1], np.int32)]
        with pytest.raises(SSError, match="needs 1 <= k <= i"):
            ctx.set_quartets(*bad)  # i < k
        with pytest.raises(SSError, match="needs 1 <= k <= i"):
            ctx.set_quartets(*[np.array([8], np.int32)] * 4)  # beyond the 7 functions


def test_order_duplicates_and_subsets():
    b = configs.h2o_26(ng0=6)
    q = [np.asarray(a) for a in basis.build_mapping(b.n)]
    rng = np.random.default_rng(3)
    sel = rng.choice(len(q[0]), 500, replace=False)
    sel = np.concatenate([sel, sel[:50]])  # duplicates
    rng.shuffle(sel)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        full, _ = ctx.gauss_eri()
        ctx.set_quartets(*[np.ascontiguousarray(a[sel]) for a in q])
        sub, _ = ctx.gauss_eri()
    np.testing.assert_allclose(sub, full[sel], rtol=1e-13, atol=1e-18)
