"""Known-answer tests that pin the CPU oracle (the reference ships no golden outputs).

* Boys-type integrals F_n(rho) = int_0^1 t^2n exp(-rho t^2) dt against adaptive quadrature in
  every regime of src/rint_sum.F90 (rho = 0, rho < 1 Taylor, 1 <= rho <= 80 recursion, rho > 80).
* s-type primitive ERI closed form 2 pi^{5/2} / (p q sqrt(p+q)) F_0(pq/(p+q) |PQ|^2) E_AB E_CD.
* p-type primitive ERIs against the derivative of the s-type closed form w.r.t. the centre.
* unnormalised STO 1s self-repulsion (1s1s|1s1s) = 5 pi^2 / (8 zeta^5), which the 20-Gaussian
  fit reproduces to ~1e-5 and the fit + ZV-MC correction must reproduce within 4 sigma.
* dierfc (src/dierfc.F90) as the inverse of erfc.
"""
import math

import numpy as np
import pytest
from scipy import integrate, special

from oracle import binding as O
from slater_stoch_gb300 import basis, configs

PI_5_2 = 34.9868366552  # the reference's 12-digit 2 pi^{5/2}


def boys_quad(n, rho):
    return integrate.quad(lambda t: t ** (2 * n) * math.exp(-rho * t * t), 0, 1, epsabs=1e-300,
                          epsrel=2e-14, limit=200)[0]


@pytest.mark.parametrize("rho", [0.0, 1e-6, 0.3, 0.999, 1.0, 2.5, 10.0, 40.0, 79.0, 85.0])
@pytest.mark.parametrize("n", [0, 1, 2, 5, 8])
def test_boys_against_quadrature(n, rho):
    v = O.rint(n, rho)
    ref = boys_quad(n, rho)
    # upward recursion (rho >= 1) loses digits for large n near rho ~ 1 (reference behaviour)
    tol = 1e-13 if (rho < 1.0 or n <= 2) else 1e-9
    assert abs(v - ref) <= tol * max(abs(ref), 1e-300) + 1e-16


def test_rint_sum_is_linear_in_d1():
    d = np.array([1.0, 0, 0.5, 0, 0.25, 0, 0.125])
    for rho in (0.0, 0.5, 3.0):
        s = O.rint_sum(6, rho, d)
        ref = sum(d[2 * k] * O.rint(k, rho) for k in range(4))
        assert abs(s - ref) <= 1e-14 * abs(ref)


def test_s_primitive_closed_form():
    A = np.array([0.0, 0.0, 0.0]); B = np.array([0.0, 1.43, 1.1])
    Cc = np.array([0.3, -0.2, 0.4]); D = np.array([1.0, 0.5, -0.7])
    a, b, c, d = 0.9, 2.3, 0.4, 1.7
    p, q = a + b, c + d
    P = (a * A + b * B) / p; Q = (c * Cc + d * D) / q
    Eab = math.exp(-a * b / p * np.sum((A - B) ** 2)); Ecd = math.exp(-c * d / q * np.sum((Cc - D) ** 2))
    T = p * q / (p + q) * np.sum((P - Q) ** 2)
    F0 = 0.5 * math.sqrt(math.pi / T) * math.erf(math.sqrt(T))
    ref = PI_5_2 / (p * q * math.sqrt(p + q)) * Eab * Ecd * F0
    z = [0, 0, 0]
    v = O.bielec_integral(a, b, c, d, A, B, Cc, D, z, z, z, z)
    assert abs(v - ref) <= 1e-13 * abs(ref)


def test_p_primitive_from_centre_derivative():
    # (x - A_x) exp(-a|r-A|^2) = (1/2a) d/dA_x exp(-a|r-A|^2): finite-difference the s integral
    A = np.array([0.1, -0.2, 0.3]); B = np.array([0.0, 1.2, 0.9])
    Cc = np.array([0.5, 0.1, -0.4]); D = Cc.copy()
    a, b, c, d = 1.3, 0.7, 0.9, 0.9
    z = [0, 0, 0]
    h = 1e-5
    Ap, Am = A.copy(), A.copy()
    Ap[0] += h; Am[0] -= h
    ds = (O.bielec_integral(a, b, c, d, Ap, B, Cc, D, z, z, z, z) -
          O.bielec_integral(a, b, c, d, Am, B, Cc, D, z, z, z, z)) / (2 * h)
    v = O.bielec_integral(a, b, c, d, A, B, Cc, D, [1, 0, 0], z, z, z)
    assert abs(v - ds / (2 * a)) <= 1e-8 * abs(v)


@pytest.mark.parametrize("zeta", [1.24, 7.66])
def test_sto_1s_self_repulsion_of_fit(zeta):
    mol = basis.molecule_bohr(["H"], [[0.0, 0.0, 0.0]])
    b = basis.build_basis(mol, {1: [("1S", zeta)]}, basis.FitParams(ng0=20))
    ob = O.OracleBasis(b)
    v = O.gauss_ijkl(ob, 0, 0, 0, 0)
    exact = 5 * math.pi ** 2 / (8 * zeta ** 5)
    assert abs(v - exact) <= 1e-4 * exact


def test_sto_1s_fit_plus_zvmc_correction():
    """analytic fit ERI + faithful ZV-MC correction = exact STO value within 4 sigma."""
    zeta = 1.0
    mol = basis.molecule_bohr(["H"], [[0.0, 0.0, 0.0]])
    b = basis.build_basis(mol, {1: [("1S", zeta)]}, basis.FitParams(ng0=3))
    ob = O.OracleBasis(b)
    q = basis.build_mapping(1)
    g = O.gauss_ijkl(ob, 0, 0, 0, 0)
    rng = np.random.default_rng(3)
    nb, npts = 10, 40 * 500
    r1 = rng.standard_normal((nb * npts, 3)); r2 = rng.standard_normal((nb * npts, 3))
    m, e = O.zvmc_faithful(ob, q, 1.8, r1, r2, nb, npts, "fp64")
    exact = 5 * math.pi ** 2 / (8 * zeta ** 5)
    assert abs(g - exact) > 10 * e[0]          # the 3-Gaussian fit alone is visibly off
    assert abs(g + m[0] - exact) <= 4 * e[0] + 1e-12


def test_dierfc_inverts_erfc():
    for y in (1e-10, 0.01, 0.5, 1.0, 1.3, 1.99):
        x = O.dierfc(y)
        assert abs(special.erfc(x) - y) <= 1e-12 * y + 1e-15


def test_reference_summation_error_is_bounded():
    """The reference accumulates ~1e7 primitive terms sequentially in FP64; the exact sum of the
    same terms differs by at most ~1e-11 relative (this bounds the oracle's own rounding)."""
    fx = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "gauss_eri_h2o_minimal_ng20.npz")
    b = configs.h2o_minimal(20)
    q = basis.build_mapping(b.n)
    pre = fx["precond"].reshape(b.n, b.n, order="F")
    i, j, k, l = [np.asarray(a) - 1 for a in q]
    scale = np.sqrt(np.abs(pre[i, k] * pre[j, l]))
    d = np.abs(fx["eri"] - fx["eri_ext"])
    assert np.all(d <= 1e-11 * np.abs(fx["eri_ext"]) + 1e-14 * scale)


def test_golden_matches_oracle_subset():
    """The committed fixture is reproducible by the oracle (spot check of a few quartets)."""
    fx = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "gauss_eri_h2o_minimal_ng20.npz")
    b = configs.h2o_minimal(20)
    q = basis.build_mapping(b.n)
    ob = O.OracleBasis(b)
    O.set_sum_mode("extended")
    for t in (0, 57, 200, 405):
        i, j, k, l = [int(a[t]) - 1 for a in q]
        v = O.gauss_ijkl(ob, i, k, j, l)
        assert abs(v - fx["eri_ext"][t]) <= 1e-15 * abs(v) + 1e-300
    O.set_sum_mode("reference")


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors (Salmon et al., SC'11 reference implementation)."""
    from oracle.cleanup import philox4x32_10
    cases = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
             ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
              (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, out in cases:
        got = philox4x32_10(*[np.uint64(v) for v in ctr], *key)
        assert tuple(int(v) for v in got) == out


def test_svd_clean_oracle_makes_psd():
    from oracle import cleanup as OC
    b = configs.h2o_minimal(4)
    q = basis.build_mapping(b.n)
    ob = O.OracleBasis(b)
    O.set_sum_mode("extended")
    g, _ = O.gauss_eri(ob, q)
    for layout in ("packed_pair", "ref_n2"):
        moy = OC.perturb_indefinite(g, q, b.n, layout, seed=1)
        W = OC.matrix_from_eris(moy, q, b.n, layout)
        assert np.linalg.eigvalsh(W).min() < -1e-8
        clean, nrem = OC.svd_clean(moy, q, b.n, layout, rank=W.shape[0], q=4)
        assert nrem > 0
        lmin = np.linalg.eigvalsh(OC.matrix_from_eris(clean, q, b.n, layout)).min()
        if layout == "packed_pair":
            assert lmin >= -1e-12
        else:
            # the reference's final 8-fold average includes the i<->k exchange, a partial
            # transpose of the <ij|kl> matrix, which does not preserve semidefiniteness: the
            # cleanup only reduces the negative part there
            assert lmin > np.linalg.eigvalsh(W).min()
        assert np.max(np.abs(clean - moy)) < 1e-3


def test_davidson_oracle():
    from oracle import cleanup as OC
    rng = np.random.default_rng(2)
    A = rng.standard_normal((60, 60))
    H = A @ A.T + np.diag(np.arange(60.0))
    ev, X = OC.davidson(H, 4, tol=1e-10)
    np.testing.assert_allclose(ev, np.linalg.eigvalsh(H)[:4], rtol=1e-8)


@pytest.mark.parametrize("zeta", [1.0, 1.7])
def test_one_electron_sto_1s_known_answers(zeta):
    """One-electron integrals of the 20-Gaussian fit of an unnormalised 1s STO e^(-zeta r) on a
    unit charge at its centre (src/one_elect.F90): S = pi/zeta^3, V = -pi/zeta^2,
    K = pi/(2 zeta), reproduced to the fit's accuracy."""
    mol = basis.molecule_bohr(["H"], [[0.0, 0.0, 0.0]])
    b = basis.build_basis(mol, {1: [("1S", zeta)]}, basis.FitParams(ng0=20))
    S, V, K = O.one_elect(O.OracleBasis(b), mol.coords, mol.charges)
    assert abs(S[0, 0] - math.pi / zeta ** 3) <= 1e-10 * math.pi / zeta ** 3
    assert abs(V[0, 0] + math.pi / zeta ** 2) <= 1e-7 * math.pi / zeta ** 2
    assert abs(K[0, 0] - math.pi / (2 * zeta)) <= 1e-7 * math.pi / (2 * zeta)


def test_one_electron_gaussian_closed_forms():
    """Two s Gaussians c e^(-a r^2) at distance R (one-Gaussian fits): overlap, kinetic and the
    attraction of a unit charge at the first centre against their closed forms."""
    mol = basis.molecule_bohr(["H", "H"], [[0.0, 0.0, 0.0], [0.0, 0.3, 0.9]])
    b = basis.build_basis(mol, {1: [("1S", 1.3)]}, basis.FitParams(ng0=1))
    ob = O.OracleBasis(b)
    S, V, K = O.one_elect(ob, mol.coords[:1], [1.0])
    a = b.g_gauss[0, 0]; c = b.c_gauss[0, 0, 0]
    R2 = 0.09 + 0.81
    p = 2 * a; mu = a * a / p
    s_ref = c * c * (math.pi / p) ** 1.5 * math.exp(-mu * R2)
    k_ref = mu * (3 - 2 * mu * R2) * s_ref
    T = p * (R2 / 4)  # P is the midpoint; the charge sits at the first centre
    f0 = 0.5 * math.sqrt(math.pi / T) * math.erf(math.sqrt(T))
    v_ref = -c * c * 2 * math.pi / p * math.exp(-mu * R2) * f0
    assert abs(S[0, 1] - s_ref) <= 1e-13 * s_ref
    assert abs(K[0, 1] - k_ref) <= 1e-12 * abs(k_ref)
    assert abs(V[0, 1] - v_ref) <= 1e-12 * abs(v_ref)


# ---- exact one-centre Slater ERIs (src/ijkl_slater_xnynzn.F90) against closed forms ----------

def _radial(l, a, b, pa, pb):
    """int int r1^pa e^(-a r1) r2^pb e^(-b r2) r<^l / r>^(l+1) dr1 dr2, exact (sympy)."""
    sp = pytest.importorskip("sympy")
    r1, r2 = sp.symbols("r1 r2", positive=True)
    inner = (sp.integrate(r2 ** (pb + l) * sp.exp(-b * r2), (r2, 0, r1)) / r1 ** (l + 1)
             + r1 ** l * sp.integrate(r2 ** pb * sp.exp(-b * r2) / r2 ** (l + 1), (r2, r1, sp.oo)))
    return sp.integrate(r1 ** pa * sp.exp(-a * r1) * inner, (r1, 0, sp.oo))


def test_monocenter_closed_forms():
    """Unnormalised one-centre STO integrals from the multipole expansion of 1/r12, with the
    radial double integrals done exactly: (1s1s|1s1s) = 5 pi^2 / (8 zeta^5); (2pz 2pz|1s 1s)
    keeps the l = 0 part (1/3) of cos^2; (2pz 2pz|2px 2px) adds the l = 2 coupling
    (2/3)(-1/3)/25; (2s 1s|2s 1s) has radial powers r^1."""
    sp = pytest.importorskip("sympy")
    z = 1.7
    v = O.ijkl_slater_xnynzn([0] * 4, [0] * 4, [0] * 4, [0] * 4, [z] * 4)
    assert abs(v / (5 * np.pi ** 2 / (8 * z ** 5)) - 1) < 1e-14
    g = [sp.Rational(17, 10), sp.Rational(13, 10), sp.Rational(9, 10), sp.Rational(11, 10)]
    gf = [float(x) for x in g]
    a, b = g[0] + g[1], g[2] + g[3]
    cases = [
        (([0, 0, 0, 0], [0, 0, 0, 0], [1, 1, 0, 0], [0, 0, 0, 0]),
         16 * sp.pi ** 2 * sp.Rational(1, 3) * _radial(0, a, b, 4, 2)),
        (([0, 0, 1, 1], [0, 0, 0, 0], [1, 1, 0, 0], [0, 0, 0, 0]),
         16 * sp.pi ** 2 * (sp.Rational(1, 9) * _radial(0, a, b, 4, 4)
                            - sp.Rational(2, 9) / 25 * _radial(2, a, b, 4, 4))),
        (([0] * 4, [0] * 4, [0] * 4, [1, 0, 1, 0]), 16 * sp.pi ** 2 * _radial(0, a, b, 3, 3)),
    ]
    for (nx, ny, nz, pw), exact in cases:
        v = O.ijkl_slater_xnynzn(nx, ny, nz, pw, gf)
        assert abs(v / float(exact) - 1) < 1e-14, (nx, ny, nz, pw, v, float(exact))


def test_monocenter_vs_gaussian_fits():
    """The 20-Gaussian fits reproduce the exact one-centre Slater ERIs of the 26-function basis
    (s, p, d and 2s-type radial powers on oxygen) to 1e-6 relative: a check of the spherical-
    harmonic coefficients of x^nx y^ny z^nz and of the fits at once."""
    b = configs.h2o_26(ng0=20)
    q = np.array(basis.build_mapping(b.n))
    ob = O.OracleBasis(b)
    ex, mask = O.monocenter(ob, q)
    assert mask.sum() == 9556
    d_fn = np.flatnonzero(b.npower.reshape(-1, 3).sum(axis=1) == 2) + 1
    idx = np.flatnonzero(mask & np.isin(q[0], d_fn) & (np.abs(ex) > 1e-6))
    sel = np.random.default_rng(3).choice(idx, 6, replace=False)
    g, _ = O.gauss_eri(ob, q[:, sel])
    assert np.all(np.abs(g - ex[sel]) <= 1e-6 * np.abs(ex[sel]))


def test_monocenter_beyond_d_refused():
    """Functions with nx+ny+nz > 2 stop the reference (src/ijkl_slater_xnynzn.F90:41-44)."""
    with pytest.raises(ValueError):
        O.ijkl_slater_xnynzn([3, 0, 0, 0], [0] * 4, [0] * 4, [0] * 4, [1.0] * 4)
