"""Workload definitions (synthetic inputs; the reference ships no benchmark data).

* ``h2o_minimal``   -- H2O, O(0,0,0), H(0,+-1.4305,1.1093) bohr; O 1s 7.66, 2s 2.25, 2p 2.25,
                       H 1s 1.24; 7 functions, 406 unique ERIs.
* ``h2o_26``        -- same geometry; O 1s 7.9/6.6, 2s 2.7/1.7, 2p 2.9/1.5, 3d 2.0;
                       H 1s 1.6/1.0, 2p 1.3; 26 functions, 61,776 unique ERIs.
* ``random_molecule`` -- seeded generator: atoms with Z uniform in {1,6,7,8}, uniform in a cube
                       with a minimum separation, heavy atoms 1s 2s 2p 3d, H 1s 2p,
                       zeta = Slater-rule value x U[0.8, 1.2].

Slater-rule exponents used by the generator (Z_eff / n): H 1s 1.0; C 1s 5.70, 2s/2p 1.625;
N 1s 6.70, 2s/2p 1.95; O 1s 7.70, 2s/2p 2.275.  Polarisation shells (3d on heavy atoms, 2p on
H) have no occupied Slater-rule value; they take the valence exponent of the same atom.
"""
from __future__ import annotations

import numpy as np

from .basis import FitParams, build_basis, molecule_bohr

H2O_BOHR = [[0.0, 0.0, 0.0], [0.0, 1.4305, 1.1093], [0.0, -1.4305, 1.1093]]


def h2o_minimal(ng0: int = 20):
    mol = molecule_bohr(["O", "H", "H"], H2O_BOHR)
    basis = {8: [("1S", 7.66), ("2S", 2.25), ("2P", 2.25)], 1: [("1S", 1.24)]}
    return build_basis(mol, basis, FitParams(ng0=ng0))


def h2o_26(ng0: int = 20):
    mol = molecule_bohr(["O", "H", "H"], H2O_BOHR)
    basis = {8: [("1S", 7.9), ("1S", 6.6), ("2S", 2.7), ("2S", 1.7), ("2P", 2.9), ("2P", 1.5),
                 ("3D", 2.0)],
             1: [("1S", 1.6), ("1S", 1.0), ("2P", 1.3)]}
    return build_basis(mol, basis, FitParams(ng0=ng0))


SLATER = {1: {"1S": 1.0, "2P": 1.0},
          6: {"1S": 5.70, "2S": 1.625, "2P": 1.625, "3D": 1.625},
          7: {"1S": 6.70, "2S": 1.95, "2P": 1.95, "3D": 1.95},
          8: {"1S": 7.70, "2S": 2.275, "2P": 2.275, "3D": 2.275}}
SYM = {1: "H", 6: "C", 7: "N", 8: "O"}


def random_molecule(seed: int, natoms: int = 12, box: float = 8.0, min_sep: float = 2.0,
                    ng0: int = 20, max_tries: int = 100000):
    """Seeded random molecule (the large single-system workload)."""
    rng = np.random.default_rng(seed)
    zs = rng.choice([1, 6, 7, 8], size=natoms)
    pos = []
    tries = 0
    while len(pos) < natoms:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place atoms with the requested separation")
        p = rng.uniform(0.0, box, size=3)
        if all(np.linalg.norm(p - q) >= min_sep for q in pos):
            pos.append(p)
    mol = molecule_bohr([SYM[int(z)] for z in zs], np.array(pos))
    # one basis list per atom: exponents are drawn per atom, so build per-atom element keys
    fns = []
    for ia, z in enumerate(zs):
        orbs = ["1S", "2P"] if z == 1 else ["1S", "2S", "2P", "3D"]
        fns.append([(o, SLATER[int(z)][o] * rng.uniform(0.8, 1.2)) for o in orbs])
    return _build_per_atom(mol, fns, FitParams(ng0=ng0))


def _build_per_atom(mol, per_atom, fit):
    """build_basis with a different exponent list per atom (same ordering rules)."""
    from .basis import Basis
    parts = []
    for ia in range(len(mol.symbols)):
        sub = molecule_bohr([mol.symbols[ia]], mol.coords[ia:ia + 1])
        z = int(mol.charges[ia])
        parts.append((ia, build_basis(sub, {z: per_atom[ia]}, fit)))
    n = sum(p.n for _, p in parts)
    ld = max(p.ld for _, p in parts)
    out = Basis(center=np.zeros((n, 3)), npower=np.zeros((n, 3), np.int32),
                n_sto=np.zeros(n, np.int32), i_type=np.zeros(n, np.int32),
                n_gauss=np.zeros(n, np.int32), c_gauss=np.zeros((2, n, ld)),
                g_gauss=np.zeros((n, ld)), g_slater=np.zeros(n), nucleus=np.zeros(n, np.int32),
                names=[], shell=np.zeros(n, np.int32))
    o = 0
    sh = 0
    for ia, p in parts:
        m = p.n
        out.center[o:o + m] = p.center
        out.npower[o:o + m] = p.npower
        out.n_sto[o:o + m] = p.n_sto
        out.i_type[o:o + m] = p.i_type
        out.n_gauss[o:o + m] = p.n_gauss
        out.c_gauss[:, o:o + m, :p.ld] = p.c_gauss
        out.g_gauss[o:o + m, :p.ld] = p.g_gauss
        out.g_slater[o:o + m] = p.g_slater
        out.nucleus[o:o + m] = ia
        out.names += [f"{mol.symbols[ia]}{ia + 1}:" + nm.split(":", 1)[1] for nm in p.names]
        out.shell[o:o + m] = p.shell + sh
        sh += int(p.shell.max()) + 1
        o += m
    return out


def batch_systems(seed: int, count: int = 512, min_atoms: int = 2, max_atoms: int = 10,
                  ng0: int = 20):
    """Many seeded small systems of uneven size (the batched workload)."""
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        na = int(rng.integers(min_atoms, max_atoms + 1))
        out.append(random_molecule(int(rng.integers(0, 2**31 - 1)), natoms=na, ng0=ng0,
                                   box=max(4.0, 8.0 * (na / 12.0) ** (1 / 3))))
    return out
