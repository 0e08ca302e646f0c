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


def _stratified(counts, cls, per_class=40, top_fp32=50, seed=20):
    """>= per_class quartets of every kernel instance (L, LK, tc) (all of a smaller class) and the
    top_fp32 quartets with the largest FP32-tier share of their kept primitive quartets."""
    rng = np.random.default_rng(seed)
    keys = cls[:, 0] * 100 + cls[:, 1] * 10 + cls[:, 2]
    sel = set()
    for key in np.unique(keys):
        idx = np.nonzero(keys == key)[0]
        sel.update(rng.choice(idx, min(per_class, idx.size), replace=False).tolist())
    kept = counts[:, 1] + counts[:, 2]
    share = np.where(kept > 0, counts[:, 1] / np.maximum(kept, 1), 0.0)
    sel.update(np.argsort(-share, kind="stable")[:top_fp32].tolist())
    return np.array(sorted(sel)), share


@pytest.fixture(scope="module")
def h2o26_ng20(tmp_path_factory):
    """The benchmarked workload: 26-function H2O basis, 20-Gaussian fits, all 61,776 quartets on
    the device (screening and the FP32 tier on); the oracle's Schwarz diagonal and the kernel's
    own tier split of every quartet (host build of the kernel arithmetic)."""
    import eri_host
    if not eri_host.available():
        pytest.fail("g++ and the CUDA headers are needed to build the kernel's host arithmetic")
    O = _oracle()
    b = configs.h2o_26(ng0=20)
    q = basis.build_mapping(b.n)
    ob = O.OracleBasis(b)
    pre = O.precond(ob)
    L = eri_host.load(eri_host.build(tmp_path_factory.mktemp("erihost")))
    return O, b, q, ob, pre, L, {}  # the last: oracle values by quartet index, shared by the cases


@pytest.mark.parametrize("fp32_eps", [1e-11, 1e-13])
def test_gauss_eri_h2o26_ng20_stratified(h2o26_ng20, fp32_eps):
    """All 61,776 ERIs of the benchmarked configuration computed on the device; compared with the
    oracle on the whole Schwarz diagonal (351 quartets (ik|ik)), a stratified sample of >= 40
    quartets from every kernel instance (L, LK, tc), and the 50 quartets whose kept primitive
    quartets go most to the FP32 tier.  Gate per quartet: 1e-12 |ERI| + 1e-12 sqrt((ik|ik)(jl|jl)).
    Run at the default FP32-tier threshold (1e-11 of the Schwarz bound) and at 1e-13."""
    import eri_host
    O, b, q, ob, pre, L, memo = h2o26_ng20
    counts, cls = eri_host.tier_counts(L, b, q, pre, 1e-18, fp32_eps)
    qa = [np.asarray(a) for a in q]
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        ctx.set_eri_tiers(1e-18, fp32_eps)
        gp = ctx.precond()
        g, nz = ctx.gauss_eri()
    np.testing.assert_allclose(gp.reshape(-1, order="F"), pre, rtol=RTOL, atol=0)
    sel, share = _stratified(counts, cls)
    sub = [a[sel] for a in qa]
    todo = np.array([t for t in sel if t not in memo], dtype=np.int64)
    if todo.size:
        vals, _ = O.gauss_eri(ob, [a[todo] for a in qa], pre)
        memo.update(zip(todo.tolist(), vals.tolist()))
    ref = np.array([memo[t] for t in sel.tolist()])
    n = b.n
    P = pre.reshape(n, n, order="F")
    i, j, k, l = [a - 1 for a in sub]
    bound = RTOL * np.abs(ref) + RTOL * np.sqrt(np.abs(P[i, k] * P[j, l]))
    ratio = _gate_ratio(np.abs(g[sel] - ref), bound)
    worst = int(np.argmax(ratio))
    print(f"\nh2o_26 ng0=20 fp32_eps={fp32_eps:g}: {sel.size} quartets vs oracle, worst |gpu-oracle|/gate "
          f"{ratio[worst]:.3e} (quartet {[int(x[worst]) for x in sub]}, FP32 share {share[sel][worst]:.2f}); "
          f"largest FP32 share in the sample {share[sel].max():.3f}")
    assert np.all(ratio <= 1.0), f"{(ratio > 1).sum()} quartets outside the gate, worst ratio {ratio.max():.3g}"


def _gate_ratio(diff, bound):
    """|gpu - oracle| / gate per quartet; a quartet with a zero gate (a pair whose Schwarz
    diagonal is exactly zero, e.g. two distant functions whose primitive pairs all vanish) must
    match exactly (ratio 0, else inf)."""
    safe = np.where(bound > 0, bound, 1.0)
    return np.where(bound > 0, diff / safe, np.where(diff == 0, 0.0, np.inf))


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


def test_gauss_eri_random_molecule_subset():
    """The large single-system workload: the seeded 12-atom random molecule (111 STOs, 20-Gaussian
    fits, 1.93e7 unique quartets).  The device computes the whole Schwarz diagonal (6,216
    quartets (ik|ik)) and the ERIs of a subset: >= 8 quartets of every kernel instance
    (L, LK, tc) and 60 more at random; the oracle computes the same quartets and the diagonal
    entries they need.  Gate per quartet: 1e-12 |ERI| + 1e-12 sqrt((ik|ik)(jl|jl))."""
    from slater_stoch_gb300 import perfmodel
    O = _oracle()
    b = configs.random_molecule(1)
    q = basis.build_mapping(b.n)
    cls = perfmodel.kernel_classes(b, q)
    rng = np.random.default_rng(12)
    keys = cls[:, 0] * 100 + cls[:, 1] * 10 + cls[:, 2]
    sel = set(rng.choice(len(keys), 60, replace=False).tolist())
    for key in np.unique(keys):
        idx = np.nonzero(keys == key)[0]
        sel.update(rng.choice(idx, min(8, idx.size), replace=False).tolist())
    sel = np.array(sorted(sel))
    sub = [np.ascontiguousarray(a[sel]) for a in q]
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*sub)
        gp = ctx.precond()
        g, _ = ctx.gauss_eri()
    ob = O.OracleBasis(b)
    pairs = sorted({(int(i), int(k)) for i, k in zip(sub[0], sub[2])} | {(int(j), int(l)) for j, l in zip(sub[1], sub[3])})
    pi = np.array([p[0] for p in pairs], np.int32)
    pk = np.array([p[1] for p in pairs], np.int32)
    diag = O.gauss_list(ob, [pi, pi, pk, pk])  # the (ik|ik) these quartets need
    pre = np.zeros((b.n, b.n))
    pre[pi - 1, pk - 1] = diag
    pre[pk - 1, pi - 1] = diag
    np.testing.assert_allclose(gp[pi - 1, pk - 1], diag, rtol=RTOL, atol=0)
    ref, _ = O.gauss_eri(ob, sub, pre.reshape(-1, order="F"))
    i, j, k, l = [a - 1 for a in sub]
    bound = RTOL * np.abs(ref) + RTOL * np.sqrt(np.abs(pre[i, k] * pre[j, l]))
    ratio = _gate_ratio(np.abs(g - ref), bound)
    print(f"\nrandom molecule (111 STOs): {sel.size} quartets of {len(keys)} vs oracle, "
          f"{len(np.unique(keys))} kernel instances, worst |gpu-oracle|/gate {ratio.max():.3e}")
    assert np.all(ratio <= 1.0), f"{(ratio > 1).sum()} quartets outside the gate, worst {ratio.max():.3g}"
