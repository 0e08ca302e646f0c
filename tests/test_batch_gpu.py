"""The batched workload (slater_stoch_gb300/batch.py): several systems of uneven size in one
basis with ss_basis_systems, their quartets in one ss_gauss_eri (one launch per kernel class
for all systems), each system's MC correction as its own concurrent job.  Each system's result
must equal the same system run alone (ss_two_e_job on a fresh context): the analytic values to
rounding (1e-13 relative: the bra-slice split of a quartet depends on how many quartets share
its class) and hence the ERIs to 1e-13 relative + 1e-17 Ha; the error bars bitwise-equivalent
to 1e-12 (same seeds, same walkers)."""
import numpy as np
import pytest

from slater_stoch_gb300 import api, basis, batch, configs
from slater_stoch_gb300._lib import SSError

pytestmark = pytest.mark.gpu


def _systems():
    rng = np.random.default_rng(4)
    out = [configs.random_molecule(int(rng.integers(1, 2 ** 31 - 1)), natoms=na, box=4.0, ng0=6)
           for na in (1, 2, 1, 2, 3)]
    out.append(configs.h2o_minimal(ng0=6))
    return out


def test_batch_equals_each_system_alone():
    systems = _systems()
    seeds = list(range(11, 11 + len(systems)))
    res, rep = batch.batch_two_e(systems, seeds, sigma_target=1e-4, npts=1 << 13, nblocks_max=8, max_running=3)
    s = rep.summary()
    assert s["systems"] == len(systems) and len(rep.latency_s) == len(systems)
    assert len(set(b.n for b in systems)) >= 3  # uneven sizes
    for b, sd, (eri, sig) in zip(systems, seeds, res):
        with api.Context(0) as ctx:
            ctx.set_basis(b)
            ctx.set_quartets(*basis.build_mapping(b.n))
            e1, s1 = ctx.two_e_job(1.8, sd, 1 << 13, 8, "shared", "split_bf16", 1e-4)
        np.testing.assert_allclose(eri, e1, rtol=1e-13, atol=1e-17)
        np.testing.assert_allclose(sig, s1, rtol=1e-12, atol=1e-17)


def test_multi_system_basis_refuses_direct_mc():
    systems = _systems()[:2]
    comb, first = batch.concat_systems(systems)
    with api.Context(0) as ctx:
        ctx.set_basis(comb)
        from slater_stoch_gb300._lib import check
        check(ctx._L.ss_basis_systems(ctx._h, 2, first))
        q = basis.build_mapping(systems[0].n)
        ctx.set_quartets(*q)
        with pytest.raises(SSError, match="several systems"):
            ctx.zvmc(1.8, 1, 4096, 2, "shared", "split_bf16")
