"""Integral output in the reference's formats (src/two_e_slater.F90:572-615).

* ``write_bielec_ao`` -- the text file ``bielec_ao``: one line per quartet,
  Fortran format ``'(4(I5,X),2D22.15)'`` with i, j, k, l (1-based, physicist <ij|kl> = (ik|jl)),
  the integral and its MC error (:605-613).
* ``trexio_chunks`` -- the sparse ``ao_2e_int_eri`` layout written through TREXIO (:574-601):
  quartets with |v| >= 1e-15, indices (i, j, k, l), in buffers of 4096 with running offsets.
  libtrexio is not available here; ``write_trexio_npz`` stores the same arrays in a .npz.
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Iterator, Tuple

import numpy as np

BUFSIZE = 4096  # src/two_e_slater.F90:78


def fortran_d(x: float, w: int = 22, d: int = 15) -> str:
    """Fortran ``Dw.d`` edit descriptor (0.ddd...D+ee), as gfortran writes it."""
    x = float(x)
    if x == 0.0 or not math.isfinite(x):
        body = "0." + "0" * d + "D+00" if x == 0.0 else ("Infinity" if x > 0 else "-Infinity")
        return body.rjust(w)
    s = f"{abs(x):.{d - 1}e}"  # d significant digits: m.mmm...e+XX
    mant, ex = s.split("e")
    digits = mant.replace(".", "")
    e10 = int(ex) + 1
    exp = f"{'+' if e10 >= 0 else '-'}{abs(e10):02d}"
    if abs(e10) > 99:  # three-digit exponents drop the letter
        exp = f"{'+' if e10 >= 0 else '-'}{abs(e10):03d}"
        body = "0." + digits + exp
    else:
        body = "0." + digits + "D" + exp
    if x < 0:
        body = "-" + body
    return body.rjust(w)


def write_bielec_ao(path, quartets, values, sigma) -> None:
    is_, js, ks, ls = quartets
    with open(path, "w") as f:
        for t in range(len(values)):
            f.write(f"{int(is_[t]):5d} {int(js[t]):5d} {int(ks[t]):5d} {int(ls[t]):5d} "
                    f"{fortran_d(values[t])}{fortran_d(sigma[t])}\n")


def write_one_e_matrix(path, M) -> None:
    """one_e_slater's '(2(I5,X),D22.15)' i,k,M(i,k) records, i outer (src/one_e_slater.F90:125-135)."""
    M = np.asarray(M)
    n = M.shape[0]
    with open(path, "w") as f:
        for i in range(n):
            for k in range(n):
                f.write(f"{i + 1:5d} {k + 1:5d} {fortran_d(M[i, k])}\n")


def read_bielec_ao(path) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    idx, val, err = [], [], []
    for line in Path(path).read_text().splitlines():
        f = line.split()
        idx.append([int(v) for v in f[:4]])
        val.append(float(f[4].replace("D", "e")))
        err.append(float(f[5].replace("D", "e")))
    return np.array(idx, np.int32), np.array(val), np.array(err)


def trexio_chunks(quartets, values) -> Iterator[Tuple[int, np.ndarray, np.ndarray]]:
    """(offset, indx(count,4), vals(count)) buffers as passed to trexio_write_ao_2e_int_eri."""
    is_, js, ks, ls = [np.asarray(a) for a in quartets]
    keep = np.abs(np.asarray(values)) >= 1e-15
    idx = np.stack([is_[keep], js[keep], ks[keep], ls[keep]], axis=1).astype(np.int32)
    vals = np.asarray(values)[keep]
    for off in range(0, len(vals), BUFSIZE):
        yield off, idx[off:off + BUFSIZE], vals[off:off + BUFSIZE]


def write_trexio_npz(path, quartets, values) -> int:
    chunks = list(trexio_chunks(quartets, values))
    idx = np.concatenate([c[1] for c in chunks]) if chunks else np.zeros((0, 4), np.int32)
    vals = np.concatenate([c[2] for c in chunks]) if chunks else np.zeros(0)
    np.savez(path, ao_2e_int_eri_indices=idx, ao_2e_int_eri_values=vals)
    return len(vals)
