"""Python mirror of the two-electron path's entry points, over the C ABI.

The reference's driver (src/two_e_slater.F90) calls, in order:
``gauss_ijkl`` for the Schwarz diagonal (:230-236) and every quartet (:264-279),
the inline ZV-MC blocks (:386-496), the merge (:558-564) and ``svd_clean`` (:565-567).
``Context`` exposes the same steps as batched GPU calls:

    ctx = Context()
    ctx.set_basis(basis); ctx.set_quartets(*build_mapping(basis.n))
    g = ctx.gauss_eri()                       # analytic Gaussian-fit ERIs
    mean, sigma = ctx.zvmc(a_zv=1.8, seed=1, npts=..., nblocks=10)
    eri = ctx.combine()                       # gauss + MC correction
    eri_psd = ctx.psd_clean(eri, rank=..., q=...)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .basis import Basis

ESTIMATORS = {"faithful": 0, "shared": 1}
PRECISIONS = {"fp64": 0, "ref32": 1, "split_bf16": 2}
LAYOUTS = {"ref_n2": 0, "packed_pair": 1}


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._L = _lib.load()
        h = self._L.ss_create(int(device), int(hbm_budget))
        if not h:
            raise _lib.SSError(-3, (self._L.ss_last_error() or b"").decode())
        self._h = C.c_void_p(h)
        self.n = 0
        self.nint = 0
        self._job_nint = {}

    # -- lifetime ------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.ss_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self._L.ss_launch_count(self._h))

    # -- setup ---------------------------------------------------------------------
    def set_basis(self, b: Basis):
        self._basis_arrays = [np.ascontiguousarray(b.center, np.float64).reshape(-1),
                              np.ascontiguousarray(b.npower, np.int32).reshape(-1),
                              np.ascontiguousarray(b.n_sto, np.int32),
                              np.ascontiguousarray(b.i_type, np.int32),
                              np.ascontiguousarray(b.n_gauss, np.int32),
                              np.ascontiguousarray(b.c_gauss, np.float64).reshape(-1),
                              np.ascontiguousarray(b.g_gauss, np.float64).reshape(-1),
                              np.ascontiguousarray(b.g_slater, np.float64)]
        a = self._basis_arrays
        _lib.check(self._L.ss_basis_set(self._h, int(b.n), a[0], a[1], a[2], a[3], a[4], a[5],
                                        int(b.ld), a[6], a[7]))
        self.n = int(b.n)

    def set_quartets(self, is_, js, ks, ls):
        q = [np.ascontiguousarray(x, np.int32) for x in (is_, js, ks, ls)]
        _lib.check(self._L.ss_quartets_set(self._h, len(q[0]), *q))
        self.nint = len(q[0])

    # -- analytic ------------------------------------------------------------------
    def precond(self) -> np.ndarray:
        out = np.zeros(self.n * self.n)
        _lib.check(self._L.ss_precond(self._h, _ptr(out)))
        return out.reshape(self.n, self.n, order="F")

    def set_eri_tiers(self, screen_eps: float = 1e-18, fp32_eps: float = 1e-11):
        """Primitive-quartet screen and FP32-tier thresholds of the analytic stage, relative to
        each quartet's Schwarz bound (ss_set_eri_tiers)."""
        _lib.check(self._L.ss_set_eri_tiers(self._h, float(screen_eps), float(fp32_eps)))

    def gauss_eri(self, copy: bool = True):
        out = np.zeros(self.nint) if copy else None
        nrem = np.zeros(1, np.int64)
        _lib.check(self._L.ss_gauss_eri(self._h, _ptr(out), _ptr(nrem)))
        return (out, int(nrem[0])) if copy else int(nrem[0])

    # -- Monte Carlo -----------------------------------------------------------------
    def zvmc(self, a_zv: float, seed: int, npts: int, nblocks: int, estimator: str = "faithful",
             precision: str = "fp64", sigma_target: float = 0.0, copy: bool = True):
        mean = np.zeros(self.nint) if copy else None
        sigma = np.zeros(self.nint) if copy else None
        _lib.check(self._L.ss_zvmc(self._h, float(a_zv), int(seed), int(npts), int(nblocks),
                                   ESTIMATORS[estimator], PRECISIONS[precision], float(sigma_target),
                                   _ptr(mean), _ptr(sigma)))
        return mean, sigma

    def zvmc_walkers(self, a_zv: float, r1, r2, npts: int, nblocks: int, precision: str = "fp64"):
        r1 = np.ascontiguousarray(r1, np.float64).reshape(-1)
        r2 = np.ascontiguousarray(r2, np.float64).reshape(-1)
        mean = np.zeros(self.nint)
        sigma = np.zeros(self.nint)
        _lib.check(self._L.ss_zvmc_walkers(self._h, float(a_zv), r1, r2, int(npts), int(nblocks),
                                           PRECISIONS[precision], _ptr(mean), _ptr(sigma)))
        return mean, sigma

    def draw_walkers(self, seed: int, first: int, S: int):
        r1 = np.zeros((S, 3))
        r2 = np.zeros((S, 3))
        _lib.check(self._L.ss_draw_walkers(self._h, int(seed), int(first), int(S), _ptr(r1), _ptr(r2)))
        return r1, r2

    def shared_samples(self, a_zv: float, seed: int, first: int, S: int):
        u1 = np.zeros((S, 3))
        u2 = np.zeros((S, 3))
        w = np.zeros(S)
        _lib.check(self._L.ss_shared_samples(self._h, float(a_zv), int(seed), int(first), int(S),
                                             _ptr(u1), _ptr(u2), _ptr(w)))
        return u1, u2, w

    def two_e_job(self, a_zv: float, seed: int, npts: int, nblocks: int, estimator: str = "shared",
                  precision: str = "split_bf16", sigma_target: float = 0.0, copy: bool = True):
        """The reference driver's whole job (src/two_e_slater.F90:219-564) recomputed on device."""
        eri = np.zeros(self.nint) if copy else None
        sig = np.zeros(self.nint) if copy else None
        _lib.check(self._L.ss_two_e_job(self._h, float(a_zv), int(seed), int(npts), int(nblocks),
                                        ESTIMATORS[estimator], PRECISIONS[precision],
                                        float(sigma_target), _ptr(eri), _ptr(sig)))
        return eri, sig

    # -- one-electron integrals -----------------------------------------------------
    def set_nuclei(self, xyz, charge):
        """Nuclei for the nuclear attraction: xyz (nat, 3) bohr, charge (nat,)."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        charge = np.ascontiguousarray(charge, np.float64).reshape(-1)
        _lib.check(self._L.ss_nuclei_set(self._h, len(charge), xyz, charge))

    def one_e(self):
        """Overlap, nuclear attraction and kinetic matrices (n x n, [i, k]) of the fits
        (src/one_e_slater.F90)."""
        n = self.n
        S = np.zeros(n * n); V = np.zeros(n * n); K = np.zeros(n * n)
        _lib.check(self._L.ss_one_e(self._h, _ptr(S), _ptr(V), _ptr(K)))
        return S.reshape(n, n, order="F"), V.reshape(n, n, order="F"), K.reshape(n, n, order="F")

    # -- exact one-centre integrals -------------------------------------------------
    def monocenter(self):
        """Exact one-centre Slater ERIs of the quartet list: (values, mask); values are 0
        where mask is False (src/compute_int_slater.F90)."""
        out = np.zeros(self.nint)
        mask = np.zeros(self.nint, np.int32)
        cnt = np.zeros(1, np.int64)
        _lib.check(self._L.ss_monocenter(self._h, _ptr(out), _ptr(mask), _ptr(cnt)))
        return out, mask.astype(bool)

    def set_exact_monocenter(self, enable: bool = True):
        """One-centre quartets take their exact value (MC error 0) in combine/two_e_job/jobs."""
        _lib.check(self._L.ss_set_exact_monocenter(self._h, int(bool(enable))))

    # -- output ----------------------------------------------------------------------
    def write_bielec_ao(self, path):
        """The reference's bielec_ao text file of the last job's merged ERIs and MC errors."""
        _lib.check(self._L.ss_write_bielec_ao(self._h, str(path).encode()))

    # -- asynchronous jobs -----------------------------------------------------------
    def job_submit(self, a_zv: float, seed: int, npts: int, nblocks: int, estimator: str = "shared",
                   precision: str = "split_bf16", sigma_target: float = 0.0) -> int:
        """Queue the job of two_e_job on a worker thread (inputs copied now); returns its id."""
        jid = np.zeros(1, np.int64)
        _lib.check(self._L.ss_job_submit(self._h, float(a_zv), int(seed), int(npts), int(nblocks),
                                         ESTIMATORS[estimator], PRECISIONS[precision],
                                         float(sigma_target), _ptr(jid)))
        self._job_nint[int(jid[0])] = self.nint
        return int(jid[0])

    def job_submit_inputs(self, b: Basis, quartets, a_zv: float, seed: int, npts: int, nblocks: int,
                          estimator: str = "shared", precision: str = "split_bf16",
                          sigma_target: float = 0.0, mc_only: bool = False) -> int:
        """Queue a job on its own system (basis b, quartet lists) without changing this
        context's basis (ss_job_submit_inputs); returns its id.  mc_only: the job returns the
        MC correction and its error bar instead of the merged ERIs (SS_JOB_MC_ONLY)."""
        a = [np.ascontiguousarray(b.center, np.float64).reshape(-1), np.ascontiguousarray(b.npower, np.int32).reshape(-1),
             np.ascontiguousarray(b.n_sto, np.int32), np.ascontiguousarray(b.i_type, np.int32),
             np.ascontiguousarray(b.n_gauss, np.int32), np.ascontiguousarray(b.c_gauss, np.float64).reshape(-1),
             np.ascontiguousarray(b.g_gauss, np.float64).reshape(-1), np.ascontiguousarray(b.g_slater, np.float64)]
        q = [np.ascontiguousarray(x, np.int32) for x in quartets]
        jid = np.zeros(1, np.int64)
        _lib.check(self._L.ss_job_submit_inputs(self._h, int(b.n), a[0], a[1], a[2], a[3], a[4], a[5], int(b.ld),
                                                a[6], a[7], len(q[0]), *q, float(a_zv), int(seed), int(npts),
                                                int(nblocks), ESTIMATORS[estimator] | (256 if mc_only else 0),
                                                PRECISIONS[precision], float(sigma_target), _ptr(jid)))
        self._job_nint[int(jid[0])] = len(q[0])
        return int(jid[0])

    def job_poll(self, job_id: int) -> bool:
        done = np.zeros(1, np.int32)
        _lib.check(self._L.ss_job_poll(self._h, int(job_id), _ptr(done)))
        return bool(done[0])

    def job_info(self, job_id: int) -> dict:
        """Of a finished job: admission wait and run time (s), MC blocks used, largest sigma."""
        w, r, m = (np.zeros(1) for _ in range(3))
        bl = np.zeros(1, np.int32)
        _lib.check(self._L.ss_job_info(self._h, int(job_id), _ptr(w), _ptr(r), _ptr(bl), _ptr(m)))
        return {"wait_s": float(w[0]), "run_s": float(r[0]), "blocks": int(bl[0]), "max_sigma": float(m[0])}

    def job_result(self, job_id: int):
        """Wait for the job; (eri, sigma).  Raises with the job's own error if it failed."""
        nint = self._job_nint.pop(int(job_id), self.nint)
        eri = np.zeros(nint)
        sig = np.zeros(nint)
        _lib.check(self._L.ss_job_result(self._h, int(job_id), _ptr(eri), _ptr(sig)))
        return eri, sig

    def job_limits(self, eri_budget_bytes: int = 0, max_running: int = 0):
        """Admit this context's jobs in submission order within an ERI-buffer budget (bytes,
        0 = none) and a number of concurrent jobs (0 = none)."""
        _lib.check(self._L.ss_job_limits(self._h, int(eri_budget_bytes), int(max_running)))

    def job_stats(self) -> dict:
        v = [np.zeros(1, np.int32) for _ in range(3)] + [np.zeros(1, np.uint64)]
        _lib.check(self._L.ss_job_stats(self._h, *[_ptr(a) for a in v]))
        return {"running": int(v[0][0]), "queued": int(v[1][0]), "peak_running": int(v[2][0]),
                "peak_bytes": int(v[3][0])}

    def job_footprint(self) -> int:
        """Device bytes of this context's quartet count by which its jobs are admitted."""
        return int(self._L.ss_job_footprint(int(self.nint)))

    def invalidate(self):
        _lib.check(self._L.ss_invalidate(self._h))

    @property
    def max_sigma(self) -> float:
        return float(self._L.ss_mc_max_sigma(self._h))

    @property
    def blocks_done(self) -> int:
        return int(self._L.ss_mc_blocks_done(self._h))

    @property
    def stream_ptr(self) -> int:
        return int(self._L.ss_stream(self._h) or 0)

    def split_bf16_gemm(self, a_hi, a_lo, b_hi, b_lo, ksplit: int = 0) -> np.ndarray:
        """C = Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T on the tensor cores; inputs (P,K) uint16 BF16 bits."""
        arrs = [np.ascontiguousarray(x, np.uint16) for x in (a_hi, a_lo, b_hi, b_lo)]
        P, K = arrs[0].shape
        out = np.zeros((P, P), np.float32)
        _lib.check(self._L.ss_split_bf16_gemm(self._h, int(P), int(K), *arrs, int(ksplit), out))
        return out

    def combine(self) -> np.ndarray:
        out = np.zeros(self.nint)
        _lib.check(self._L.ss_combine(self._h, _ptr(out)))
        return out

    # -- cleanup -------------------------------------------------------------------
    def psd_clean(self, moy, layout: str = "ref_n2", rank: int = 512, oversample: int = 0,
                  q: int = 12, seed: int = 1):
        moy = np.array(moy, dtype=np.float64, copy=True)
        nrem = np.zeros(1, np.int32)
        _lib.check(self._L.ss_psd_clean(self._h, moy, LAYOUTS[layout], int(rank), int(oversample),
                                        int(q), int(seed), _ptr(nrem)))
        return moy, int(nrem[0])

    def psd_project(self, moy, layout: str = "packed_pair"):
        """Exact removal of negative eigencomponents (davidson_clean's small-basis path)."""
        moy = np.array(moy, dtype=np.float64, copy=True)
        nrem = np.zeros(1, np.int32)
        _lib.check(self._L.ss_psd_project(self._h, moy, LAYOUTS[layout], _ptr(nrem)))
        return moy, int(nrem[0])

    def davidson_clean(self, moy, layout: str = "ref_n2", block: int = 0, max_blocks: int = 0,
                       tol: float = 1e-8, max_iter: int = 2000):
        """Matrix-free removal of negative eigencomponents (davidson_clean's nbasis >= 200 path)."""
        moy = np.array(moy, dtype=np.float64, copy=True)
        nrem = np.zeros(1, np.int32)
        _lib.check(self._L.ss_davidson_clean(self._h, moy, LAYOUTS[layout], int(block), int(max_blocks),
                                             float(tol), int(max_iter), _ptr(nrem)))
        return moy, int(nrem[0])

    def davidson(self, moy, m: int = 10, layout: str = "packed_pair", tol: float = 1e-8,
                 max_iter: int = 200):
        moy = np.ascontiguousarray(moy, np.float64)
        N = self.n * (self.n + 1) // 2 if layout == "packed_pair" else self.n * self.n
        ev = np.zeros(m)
        vec = np.zeros((m, N))
        _lib.check(self._L.ss_davidson(self._h, moy, LAYOUTS[layout], int(m), float(tol), int(max_iter),
                                       _ptr(ev), _ptr(vec)))
        return ev, vec.T


def write_one_e_ao(directory, S, V, K):
    """one_e_slater's text outputs overlap_ao_ex, nuclear_ao_ex, kinetic_ao_ex (n x n, [i, k]),
    written by the library."""
    from pathlib import Path
    L = _lib.load()
    for name, M in (("overlap_ao_ex", S), ("nuclear_ao_ex", V), ("kinetic_ao_ex", K)):
        M = np.asarray(M, dtype=np.float64)
        flat = np.ascontiguousarray(M.reshape(-1, order="F"))
        _lib.check(L.ss_write_one_e_matrix(str(Path(directory) / name).encode(), int(M.shape[0]), flat))


def write_bielec_ao_arrays(path, quartets, eri, sigma=None):
    """bielec_ao text file of caller arrays, written by the library (no device needed)."""
    L = _lib.load()
    q = [np.ascontiguousarray(x, np.int32) for x in quartets]
    eri = np.ascontiguousarray(eri, np.float64)
    sig = None if sigma is None else np.ascontiguousarray(sigma, np.float64)
    _lib.check(L.ss_write_bielec_ao_arrays(str(path).encode(), len(eri), *q, eri, _ptr(sig)))
