"""One-electron integrals of the fits on the GPU (ss_one_e) vs the CPU oracle's restatement of
src/one_elect.F90 (overlap, nuclear attraction, kinetic), and the 1s STO known answers.

Tolerance: per element |gpu - oracle| <= 1e-12 |oracle| + 1e-14 max|matrix| (both sum the same
primitive terms in FP64, in different orders).
"""
import math

import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, configs

pytestmark = pytest.mark.gpu


def _mol():
    return basis.molecule_bohr(["O", "H", "H"], configs.H2O_BOHR)


@pytest.mark.parametrize("cfg,ng0", [("h2o_minimal", 20), ("h2o_26", 20), ("h2o_26", 6)])
def test_one_e_vs_oracle(cfg, ng0):
    from oracle import binding as O
    b = getattr(configs, cfg)(ng0=ng0)
    mol = _mol()
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_nuclei(mol.coords, mol.charges)
        S, V, K = ctx.one_e()
    Sr, Vr, Kr = O.one_elect(O.OracleBasis(b), mol.coords, mol.charges)
    for got, ref in ((S, Sr), (V, Vr), (K, Kr)):
        tol = 1e-12 * np.abs(ref) + 1e-14 * np.abs(ref).max()
        assert np.all(np.abs(got - ref) <= tol), np.max(np.abs(got - ref) / (np.abs(ref) + 1e-300))
    assert np.allclose(S, S.T, rtol=1e-12, atol=1e-14)  # the overlap is symmetric


def test_one_e_sto_1s():
    zeta = 1.3
    mol = basis.molecule_bohr(["H"], [[0.0, 0.0, 0.0]])
    b = basis.build_basis(mol, {1: [("1S", zeta)]}, basis.FitParams(ng0=20))
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_nuclei(mol.coords, mol.charges)
        S, V, K = ctx.one_e()
    assert abs(S[0, 0] - math.pi / zeta ** 3) <= 1e-10 * math.pi / zeta ** 3
    assert abs(V[0, 0] + math.pi / zeta ** 2) <= 1e-7 * math.pi / zeta ** 2
    assert abs(K[0, 0] - math.pi / (2 * zeta)) <= 1e-7 * math.pi / (2 * zeta)
