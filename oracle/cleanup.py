"""CPU oracle of the PSD cleanup and Davidson (TEST INFRASTRUCTURE: tests and the CPU
baseline only).  numpy restatements of the reference:

* ``svd_clean``  -- src/svd_clean.F90:1-426 (single rank): scatter of the 8 permutations,
  passes of a randomized SVD with Householder QR (ortho_qr.F90) and dgesvd (svd.F90), the
  sign test, deflation of W_work, removal of negative components from W, 8-fold average.
  The Gaussian test matrices are drawn from the same Philox4x32-10 stream as the GPU
  (``philox4x32_10`` below, Salmon et al. SC'11), so both sides project on the same
  subspaces; the reference's Fortran random_number stream cannot be reproduced.
* ``davidson``   -- src/davidson.F90:1-158 with the generalized projected problem (dsygv).

Parity status: parity unpinned (the reference's LAPACK/BLAS are unpinned and it cannot be run
here); the gates are PSD-ness and agreement with numpy's eigensolvers.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

M0, M1, W0, W1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57), 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)
STREAM_SVD = 0x53564443


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 on uint64 arrays holding 32-bit values."""
    c = [np.asarray(x, np.uint64) & MASK for x in (c0, c1, c2, c3)]
    k0, k1 = int(k0) & 0xFFFFFFFF, int(k1) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ np.uint64(k0), lo1, hi0 ^ c[3] ^ np.uint64(k1), lo0]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c


def u01_open(hi, lo):
    b = ((hi << np.uint64(32)) | lo) >> np.uint64(11)
    return (b.astype(np.float64) + 0.5) * 2.0 ** -53


def gaussian_matrix(seed: int, pas: int, N: int, r: int, tag: int = STREAM_SVD) -> np.ndarray:
    """N x r normal matrix with unit columns (src/svd_clean.F90:159-171), Philox Box-Muller."""
    idx = (np.arange(r, dtype=np.uint64)[None, :] * np.uint64(N) + np.arange(N, dtype=np.uint64)[:, None])
    c = philox4x32_10(idx & MASK, idx >> np.uint64(32), np.full(idx.shape, pas, np.uint64),
                      np.full(idx.shape, tag, np.uint64), seed & 0xFFFFFFFF, seed >> 32)
    u1, u2 = u01_open(c[0], c[1]), u01_open(c[2], c[3])
    P = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return P / np.linalg.norm(P, axis=0)[None, :]


def _perms(i, j, k, l):
    return [(i, j, k, l), (k, j, i, l), (k, l, i, j), (i, l, k, j),
            (j, i, l, k), (j, k, l, i), (l, k, j, i), (l, i, j, k)]


def matrix_from_eris(moy, quartets, n, layout="ref_n2"):
    is_, js, ks, ls = [np.asarray(a) - 1 for a in quartets]
    if layout == "ref_n2":
        N = n * n
        W = np.zeros((N, N))
        for t in range(8):
            a, b, c, d = _perms(is_, js, ks, ls)[t]
            W[a + b * n, c + d * n] = moy
    else:
        N = n * (n + 1) // 2
        W = np.zeros((N, N))
        p1 = is_ * (is_ + 1) // 2 + ks
        p2 = js * (js + 1) // 2 + ls
        W[p1, p2] = moy
        W[p2, p1] = moy
    return W


def eris_from_matrix(W, quartets, n, layout="ref_n2"):
    is_, js, ks, ls = [np.asarray(a) - 1 for a in quartets]
    if layout == "ref_n2":
        v = np.zeros(len(is_))
        for t in range(8):
            a, b, c, d = _perms(is_, js, ks, ls)[t]
            v = v + W[a + b * n, c + d * n] * 0.125
        return v
    p1 = is_ * (is_ + 1) // 2 + ks
    p2 = js * (js + 1) // 2 + ls
    return 0.5 * (W[p1, p2] + W[p2, p1])


def perturb_indefinite(moy, quartets, n, layout, seed=1, floor=1e-6):
    """ERIs plus seeded symmetric noise large enough to give the matrix negative eigenvalues
    (the effect MC noise has on a matrix whose smallest eigenvalue is small)."""
    W = matrix_from_eris(moy, quartets, n, layout)
    ev = np.linalg.eigvalsh(W)
    lam = max(ev[ev > 1e-10].min() if np.any(ev > 1e-10) else 0.0, floor)
    noise = np.random.default_rng(seed).standard_normal(len(moy))
    sigma = max(floor, 1.5 * lam / np.sqrt(W.shape[0]))
    for _ in range(40):
        out = moy + sigma * noise
        if np.linalg.eigvalsh(matrix_from_eris(out, quartets, n, layout)).min() < -1e-8:
            return out
        sigma *= 1.5
    raise RuntimeError("could not make the matrix indefinite")


def svd_clean(moy, quartets, n, layout="ref_n2", rank=512, oversample=0, q=12, seed=1):
    """Returns (cleaned ERIs, number of removed negative components)."""
    W_work = matrix_from_eris(moy, quartets, n, layout)
    W = W_work.copy()
    N = W.shape[0]
    r = min(rank + oversample, N)
    npass, removed, pas = 0, 0, 0
    while npass < N:
        P = gaussian_matrix(seed, pas, N, r)
        Z = np.linalg.qr(W_work @ P)[0]
        for _ in range(q):
            P = W_work.T @ Z
            Z = np.linalg.qr(W_work @ P)[0]
        Y = Z.T @ W_work
        UY, D, Vt = np.linalg.svd(Y, full_matrices=False)
        U = Z @ UY
        npass += r
        rk = np.einsum("ik,ki->k", U, Vt)
        D = np.where(rk < 0, -D, D)
        bad = np.abs(rk) < 0.99
        D = np.where(bad, 0.0, D)
        npass -= int(bad.sum())
        W_work -= (U * np.abs(D)[None, :]) @ Vt
        neg = D < 0
        if neg.any():
            W += (U[:, neg] * D[neg][None, :]) @ Vt[neg]
            removed += int(neg.sum())
        if np.max(np.abs(D)) < 1e-12:
            npass = N
        pas += 1
    return eris_from_matrix(W, quartets, n, layout), removed


def psd_project(moy, quartets, n, layout="packed_pair"):
    """src/davidson_clean.F90:30-116 (nbasis < 200 path): dsyev, subtract the negative
    eigencomponents, read the canonical entries back.  Returns (ERIs, number removed)."""
    W = matrix_from_eris(moy, quartets, n, layout)
    E, U = np.linalg.eigh(W)
    neg = E < 0.0
    W = W - (U[:, neg] * E[neg][None, :]) @ U[:, neg].T
    is_, js, ks, ls = [np.asarray(a) - 1 for a in quartets]
    if layout == "ref_n2":
        out = W[is_ + js * n, ks + ls * n]
    else:
        out = W[is_ * (is_ + 1) // 2 + ks, js * (js + 1) // 2 + ls]
    return out, int(neg.sum())


def davidson(H, m, tol=1e-8, max_iter=200, seed=1):
    """Lowest m eigenpairs of dense symmetric H (src/davidson.F90)."""
    n = H.shape[0]
    nmax = max(2, min(10, n // m))
    Hd = np.diag(H).copy()
    U = np.zeros((n, nmax * m))
    U[:, :m] = np.linalg.qr(gaussian_matrix(seed, 0x44415649 & 0xFFFFFFFF, n, m))[0]
    Wm = np.zeros_like(U)
    total = 0
    while total < max_iter:
        for it in range(1, nmax):
            shift = m * (it - 1)
            Wm[:, shift:shift + m] = H @ U[:, shift:shift + m]
            k = shift + m
            hs = U[:, :k].T @ Wm[:, :k]
            ss = U[:, :k].T @ U[:, :k]
            E, v = scipy.linalg.eigh(0.5 * (hs + hs.T), 0.5 * (ss + ss.T))
            X = U[:, :k] @ v[:, :m]
            WX = Wm[:, :k] @ v[:, :m]
            C = (E[None, :m] * X - WX) / np.maximum(Hd[:, None] - E[None, :m], 1e-2)
            nrm = np.linalg.norm(C, axis=0)
            total += 1
            if nrm.max() < tol:
                return E[:m], X
            if it == nmax - 1 or total >= max_iter:
                break
            U[:, k:k + m] = C / nrm[None, :]
        U[:, :m] = X
    raise RuntimeError("davidson did not converge")
