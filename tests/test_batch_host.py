"""The batched workload's host side: systems concatenated into one basis keep every function's
arrays, the system boundaries are 1-based first functions, and each system's quartets shifted by
its offset stay inside its own functions (so no quartet of the concatenated list spans two
systems)."""
import numpy as np

from slater_stoch_gb300 import basis, batch, configs


def test_concat_systems_layout():
    systems = [configs.h2o_minimal(ng0=3), configs.random_molecule(5, natoms=2, box=4.0, ng0=4),
               configs.random_molecule(9, natoms=1, box=4.0, ng0=3)]
    comb, first = batch.concat_systems(systems)
    assert first[0] == 1 and first[-1] == comb.n + 1 and len(first) == len(systems) + 1
    for s, b in enumerate(systems):
        lo, hi = first[s] - 1, first[s + 1] - 1
        assert hi - lo == b.n
        np.testing.assert_array_equal(comb.center[lo:hi], b.center)
        np.testing.assert_array_equal(comb.npower[lo:hi], b.npower)
        np.testing.assert_array_equal(comb.i_type[lo:hi], b.i_type)
        np.testing.assert_array_equal(comb.n_gauss[lo:hi], b.n_gauss)
        np.testing.assert_array_equal(comb.c_gauss[:, lo:hi, :b.ld], b.c_gauss)
        np.testing.assert_array_equal(comb.g_gauss[lo:hi, :b.ld], b.g_gauss)
        assert np.all(comb.g_gauss[lo:hi, b.ld:] == 0.0)
        q = [np.asarray(x) + lo for x in basis.build_mapping(b.n)]
        for x in q:
            assert x.min() >= lo + 1 and x.max() <= hi
