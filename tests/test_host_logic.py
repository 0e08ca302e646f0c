"""Host-side logic: input readers, basis construction, quartet map, C-ABI surface (no GPU)."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from slater_stoch_gb300 import basis, configs, perfmodel

ROOT = Path(__file__).resolve().parent.parent


def test_fit_table_complete():
    c, g = basis.load_fit_tables()
    for n in range(1, 31):
        assert np.all(c[n, 1:n + 1] != 0) and np.all(g[n, 1:n + 1] > 0)
    # SMILES 1-Gaussian fit of exp(-r) (first entry of the table)
    assert c[1, 1] == 0.7709254 and g[1, 1] == 0.6070177


@pytest.mark.parametrize("n", [1, 2, 3, 7, 26])
def test_mapping_count_and_order(n):
    is_, js, ks, ls = basis.build_mapping(n)
    P = n * (n + 1) // 2
    assert len(is_) == P * (P + 1) // 2
    assert np.all(is_ >= ks) and np.all(js >= ls) and np.all(is_ >= js)
    assert not np.any((is_ == js) & (ls > ks))
    # every unordered pair-of-pairs appears exactly once
    seen = set()
    for i, j, k, l in zip(is_, js, ks, ls):
        a, b = (int(i), int(k)), (int(j), int(l))
        key = (min(a, b), max(a, b))
        assert key not in seen
        seen.add(key)


def test_configs_sizes():
    b1 = configs.h2o_minimal()
    b2 = configs.h2o_26()
    assert b1.n == 7 and b2.n == 26
    assert perfmodel.primitive_quartets(b1, basis.build_mapping(7)) == pytest.approx(1.968e8, rel=1e-3)
    assert perfmodel.primitive_quartets(b2, basis.build_mapping(26)) == pytest.approx(1.78253e10, rel=1e-4)
    b3 = configs.random_molecule(seed=3)
    assert 50 <= b3.n <= 132


def test_basis_fit_coefficients_type2():
    # 2S: c2 = 2 c_fit g_fit zeta, g = zeta^2 g_fit (src/build_c_g_gauss_STO.F90:16-26)
    c, g = basis.load_fit_tables()
    b = configs.h2o_minimal(ng0=20)
    i = b.names.index("O1:2S")
    z = 2.25
    np.testing.assert_allclose(b.c_gauss[1, i, :20], 2 * c[20, 1:21] * g[20, 1:21] * z, rtol=0, atol=0)
    np.testing.assert_allclose(b.g_gauss[i, :20], z * z * g[20, 1:21], rtol=0, atol=0)
    assert b.i_type[i] == 2 and np.all(b.c_gauss[0, i] == 0)


def test_read_inputs(tmp_path):
    (tmp_path / "h2o.xyz").write_text("3\nWater\nO 0. 0. 0.\nH 0.0 0.756988 0.587016\nH 0.0 -0.756988 0.587016\n")
    (tmp_path / "VB").write_text("H 1S 1.24\nO 1S 7.66\nO 2S 2.25\nO 2P 2.25\n")
    (tmp_path / "j_in").write_text("Simulation number\n1\nMolecule\nh2o\nbasis\nVB\nNg\n 20 0 0 1.d30 0\n"
                                   "npts\n 4000\n****\nZV\n1.8\n")
    cfg = basis.read_j_in(tmp_path / "j_in")
    assert cfg["npts_two_elec"] == 4000 and cfg["a_zv"] == 1.8 and cfg["fit"].ng0 == 20
    mol = basis.read_geometry(tmp_path / "h2o.xyz")
    np.testing.assert_allclose(mol.coords[1], [0.0, 1.4305, 1.1093], atol=2e-5)
    b = basis.build_basis(mol, basis.read_basis(tmp_path / "VB"), cfg["fit"])
    assert b.n == 7


def test_j_in_rejects_npts_not_multiple_of_nw(tmp_path):
    (tmp_path / "j_in").write_text("t\n1\nt\nh2o\nt\nVB\nt\n 4 0 0 4. 0\nt\n 4001\nt\nt\n1.8\n")
    with pytest.raises(ValueError):
        basis.read_j_in(tmp_path / "j_in")


def test_unknown_atom_rejected():
    with pytest.raises(ValueError):
        basis.element_number("Xx")


def test_header_symbols_exported():
    """libslaterstoch.so (built for sm_103a here by nvcc) exports every function of the header."""
    from slater_stoch_gb300 import build
    lib = build.build()
    hdr = (ROOT / "include" / "slaterstoch.h").read_text()
    decl = set(re.findall(r"\b(ss_[a-z0-9_]+)\s*\(", hdr))
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ss_[a-z0-9_]+)\b", out))
    assert decl and decl <= exported, decl - exported
    from slater_stoch_gb300 import _lib
    assert set(_lib.SIGNATURES) == decl


def test_library_loads_without_gpu():
    """The ABI loads on a GPU-less host and reports the missing device instead of crashing."""
    from slater_stoch_gb300 import _lib
    L = _lib.load()
    h = L.ss_create(0, 0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert not h and L.ss_last_error()
    elif h:
        L.ss_destroy(h)


def test_fortran_d_format():
    from slater_stoch_gb300.output import fortran_d
    assert fortran_d(0.0218344660055154) == " 0.218344660055154D-01"
    assert fortran_d(-2.5) == "-0.250000000000000D+01"
    assert fortran_d(0.0) == " 0.000000000000000D+00"
    assert fortran_d(1.0) == " 0.100000000000000D+01"
    assert len(fortran_d(-1.234e-20)) == 22


def test_bielec_ao_round_trip(tmp_path):
    from slater_stoch_gb300.output import read_bielec_ao, trexio_chunks, write_bielec_ao
    q = basis.build_mapping(7)
    rng = np.random.default_rng(0)
    v = rng.standard_normal(len(q[0])) * 10.0 ** rng.integers(-20, 1, len(q[0]))
    s = np.abs(rng.standard_normal(len(q[0]))) * 1e-9
    write_bielec_ao(tmp_path / "bielec_ao", q, v, s)
    idx, vv, ss = read_bielec_ao(tmp_path / "bielec_ao")
    np.testing.assert_array_equal(idx, np.stack(q, axis=1))
    np.testing.assert_allclose(vv, v, rtol=1e-14)
    np.testing.assert_allclose(ss, s, rtol=1e-14)
    line = (tmp_path / "bielec_ao").read_text().splitlines()[0]
    assert len(line) == 4 * 6 + 2 * 22
    chunks = list(trexio_chunks(q, v))
    assert sum(len(c[2]) for c in chunks) == int(np.sum(np.abs(v) >= 1e-15))


def test_library_bielec_ao_writer_matches_fortran_format(tmp_path):
    """The library's bielec_ao writer (no device involved) produces the same bytes as the
    Fortran-format reference implementation of '(4(I5,X),2D22.15)' in output.py."""
    from slater_stoch_gb300 import api, output
    rng = np.random.default_rng(4)
    q = basis.build_mapping(5)
    nint = len(q[0])
    v = rng.standard_normal(nint) * 10.0 ** rng.integers(-120, 3, nint)
    v[:4] = [0.0, -1.0, 1.0e-100, -9.99999999999999999e-16]
    s = np.abs(rng.standard_normal(nint)) * 1e-7
    api.write_bielec_ao_arrays(tmp_path / "lib.txt", q, v, s)
    output.write_bielec_ao(tmp_path / "py.txt", q, v, s)
    assert (tmp_path / "lib.txt").read_bytes() == (tmp_path / "py.txt").read_bytes()


def test_corrupt_inputs_rejected(tmp_path):
    """Malformed inputs stop with an error instead of reaching the device: a non-numeric or
    non-positive Slater exponent, an orbital the fit builder does not know, a geometry file with
    fewer atoms than it announces."""
    mol = basis.molecule_bohr(["O"], [[0.0, 0.0, 0.0]])
    (tmp_path / "bad_zeta").write_text("O 1S seven\n")
    with pytest.raises(ValueError):
        basis.read_basis(tmp_path / "bad_zeta")
    for bad in ({8: [("1S", -1.0)]}, {8: [("1S", float("nan"))]}, {8: [("6H", 1.0)]}):
        with pytest.raises(ValueError):
            basis.build_basis(mol, bad, basis.FitParams(ng0=4))
    (tmp_path / "short.xyz").write_text("3\nWater\nO 0. 0. 0.\nH 0.0 0.75 0.58\n")
    with pytest.raises(ValueError):
        basis.read_geometry(tmp_path / "short.xyz")


def test_multi_center_counts():
    """count_multi_center_integrals: the 26-function H2O list splits into 1-, 2-, 3- and
    4-centre quartets that add up to nint; the one-centre count is the exact one-centre path's."""
    from oracle import binding as O
    b = configs.h2o_26(ng0=3)
    q = basis.build_mapping(b.n)
    c = basis.count_multi_center(b, q)
    assert sum(c.values()) == len(q[0]) and c[4] == 0  # three atoms
    _, mask = O.monocenter(O.OracleBasis(b), q)
    assert c[1] == int(mask.sum()) == 9556


def test_library_one_e_writer_matches_fortran_format(tmp_path):
    """The library's one-electron matrix files (overlap_ao_ex, nuclear_ao_ex, kinetic_ao_ex of
    one_e_slater) are byte-identical to the '(2(I5,X),D22.15)' records written by output.py."""
    from slater_stoch_gb300 import api, output
    rng = np.random.default_rng(5)
    n = 9
    mats = [rng.standard_normal((n, n)) * 10.0 ** rng.integers(-110, 3, (n, n)) for _ in range(3)]
    mats[0][0, 0] = 0.0
    api.write_one_e_ao(tmp_path, *mats)
    for name, M in zip(("overlap_ao_ex", "nuclear_ao_ex", "kinetic_ao_ex"), mats):
        output.write_one_e_matrix(tmp_path / (name + ".py"), M)
        assert (tmp_path / name).read_bytes() == (tmp_path / (name + ".py")).read_bytes()


def test_build_mapping_matches_reference_loops():
    """The vectorised quartet map equals the reference's four nested loops
    (src/build_mapping_ijkl.F90:24-43) element by element, order included."""
    for n in (1, 2, 3, 4, 7, 13):
        a = basis.build_mapping(n)
        b = basis.build_mapping_loops(n)
        assert all(np.array_equal(x, y) for x, y in zip(a, b)), n
