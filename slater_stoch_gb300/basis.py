"""STO basis construction and the unique-quartet map.

Host-side mirror of the reference's input layer (scemama/slater_stoch):

* ``read_geometry``   -- ``src/read_geometry.F90:1-41`` (xyz in angstrom -> bohr, E_nuc)
* ``read_basis``      -- ``src/read_basis.F90:1-66`` (``ATOM ORB zeta`` lines)
* ``build_basis``     -- ``src/build_gaussian_expansion_of_orbitals.F90:1-473`` and
  ``src/build_c_g_gauss_STO.F90:1-31`` (one fitted function per cartesian component)
* ``build_mapping``   -- ``src/build_mapping_ijkl.F90:9-44`` (unique (ik|jl) list)
* ``read_j_in``       -- the positional input file of ``src/two_e_slater.F90:101-154``

Array layouts are chosen so that numpy C-order arrays have the reference's
Fortran column-major memory layout (the layout of the C ABI):
``center`` (n,3) == center(3,n); ``c_gauss`` (2,n,ld) == c_gauss(ld,n,2);
``g_gauss`` (n,ld) == g_gauss(ld,n).
"""
from __future__ import annotations

import dataclasses
from pathlib import Path
from typing import Dict, List, Sequence, Tuple

import numpy as np

ANG_TO_BOHR = 1.0 / 0.52917721092  # src/read_geometry.F90:6

# src/number_atom.F90:4-8
ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P",
            "S", "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu",
            "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"]

NG_MAX = 30  # src/common_data.F90:7

# cartesian components in the reference's order
_P = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
_D = [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)]
_F = [(3, 0, 0), (2, 1, 0), (2, 0, 1), (1, 2, 0), (1, 1, 1), (1, 0, 2), (0, 3, 0), (0, 2, 1),
      (0, 1, 2), (0, 0, 3)]
_G = [(4, 0, 0), (3, 1, 0), (2, 2, 0), (1, 3, 0), (0, 4, 0), (3, 0, 1), (2, 1, 1), (1, 2, 1),
      (0, 3, 1), (2, 0, 2), (1, 1, 2), (0, 2, 2), (1, 0, 3), (0, 1, 3), (0, 0, 4)]
# orbital label -> (n_STO, i_type, components, extra Gaussians key)
ORBITALS = {
    "1S": (0, 1, [(0, 0, 0)], None),
    "2S": (1, 2, [(0, 0, 0)], None),
    "3S": (2, 2, [(0, 0, 0)], None),  # fitted as r e^-zr, evaluated as r^2 e^-zr (reference as is)
    "2P": (0, 1, _P, "2p"),
    "3P": (1, 2, _P, "2p"),
    "3D": (0, 1, _D, "3d"),
    "4F": (0, 1, _F, "3d"),
    "5G": (0, 1, _G, "3d"),
}


def element_number(sym: str) -> int:
    """``number_atom`` (src/number_atom.F90:1-18); raises on unknown symbols."""
    s = sym.strip()
    s = s[:1].upper() + s[1:].lower()
    if s not in ELEMENTS:
        raise ValueError(f"Atom not defined: {sym!r}")
    return ELEMENTS.index(s) + 1


def load_fit_tables() -> Tuple[np.ndarray, np.ndarray]:
    """SMILES STO-nG fits: c_fit[n, m], g_fit[n, m] (1-based n, m; src/read_fit_SMILES.F90)."""
    path = Path(__file__).with_name("data") / "sto_fits.txt"
    c = np.zeros((NG_MAX + 1, NG_MAX + 1))
    g = np.zeros((NG_MAX + 1, NG_MAX + 1))
    for line in path.read_text().splitlines():
        if not line.strip() or line.startswith("#"):
            continue
        n, m, cv, gv = line.split()
        c[int(n), int(m)] = float(cv)
        g[int(n), int(m)] = float(gv)
    return c, g


@dataclasses.dataclass
class Molecule:
    symbols: List[str]
    coords: np.ndarray  # (nat, 3) bohr
    charges: np.ndarray  # (nat,)

    @property
    def enucl(self) -> float:
        """Nuclear repulsion (src/read_geometry.F90:31-40)."""
        e = 0.0
        for i in range(len(self.symbols)):
            for j in range(i + 1, len(self.symbols)):
                d = self.coords[i] - self.coords[j]
                rij = np.sqrt((d[0]) ** 2 + (d[1]) ** 2 + (d[2]) ** 2)
                e += self.charges[i] * self.charges[j] / rij
        return float(e)


def read_geometry(path: str | Path) -> Molecule:
    """xyz file in angstrom -> bohr (src/read_geometry.F90:12-27)."""
    lines = Path(path).read_text().splitlines()
    nat = int(lines[0].split()[0])
    syms, xyz = [], []
    for ln in lines[2:2 + nat]:
        f = ln.split()
        syms.append(f[0])
        xyz.append([float(v) * ANG_TO_BOHR for v in f[1:4]])
    if len(syms) != nat:
        raise ValueError(f"{path}: expected {nat} atoms, found {len(syms)}")
    return Molecule(syms, np.array(xyz, dtype=np.float64),
                    np.array([element_number(s) for s in syms], dtype=np.float64))


def molecule_bohr(symbols: Sequence[str], coords_bohr) -> Molecule:
    return Molecule(list(symbols), np.asarray(coords_bohr, dtype=np.float64).reshape(-1, 3),
                    np.array([element_number(s) for s in symbols], dtype=np.float64))


def read_basis(path: str | Path) -> Dict[int, List[Tuple[str, float]]]:
    """``ATOM ORB zeta`` lines -> {Z: [(orb, zeta), ...]} (src/read_basis.F90:28-37)."""
    out: Dict[int, List[Tuple[str, float]]] = {}
    for ln in Path(path).read_text().splitlines():
        f = ln.split()
        if len(f) < 3:
            continue
        out.setdefault(element_number(f[0]), []).append((f[1].upper(), float(f[2])))
    return out


@dataclasses.dataclass
class FitParams:
    """``ng0 i_add_2p i_add_3d g_thr i_add_large_g`` (src/two_e_slater.F90:142)."""
    ng0: int = 20
    i_add_2p: int = 0
    i_add_3d: int = 0
    g_thr: float = 1.0e30
    i_add_large_g: int = 0


@dataclasses.dataclass
class Basis:
    center: np.ndarray    # (n,3) float64, bohr
    npower: np.ndarray    # (n,3) int32
    n_sto: np.ndarray     # (n,) int32
    i_type: np.ndarray    # (n,) int32
    n_gauss: np.ndarray   # (n,) int32
    c_gauss: np.ndarray   # (2,n,ld) float64
    g_gauss: np.ndarray   # (n,ld) float64
    g_slater: np.ndarray  # (n,) float64
    nucleus: np.ndarray   # (n,) int32, 0-based atom index
    names: List[str]
    shell: np.ndarray     # (n,) int32, functions sharing center, zeta and fit

    @property
    def n(self) -> int:
        return int(self.center.shape[0])

    @property
    def ld(self) -> int:
        return int(self.g_gauss.shape[1])


def build_basis(mol: Molecule, basis: Dict[int, List[Tuple[str, float]]],
                fit: FitParams = FitParams()) -> Basis:
    """One fitted function per cartesian component, in the reference's order
    (src/build_gaussian_expansion_of_orbitals.F90:11-469)."""
    c_fit, g_fit = load_fit_tables()
    rows = []
    shell_id = 0
    for ia, sym in enumerate(mol.symbols):
        Z = element_number(sym)
        for orb, zeta in basis.get(Z, []):
            if orb not in ORBITALS:
                raise ValueError(f"orbital {orb} is not supported by the fit builder")
            if not (zeta > 0.0 and np.isfinite(zeta)):
                raise ValueError(f"{sym} {orb}: Slater exponent {zeta} must be positive and finite")
            nsto, itype, comps, extra = ORBITALS[orb]
            ng = fit.ng0
            if extra == "2p":
                ng += fit.i_add_2p
            elif extra == "3d":
                ng += fit.i_add_3d
            if zeta > fit.g_thr:
                ng += fit.i_add_large_g
            if not (1 <= ng <= NG_MAX):
                raise ValueError(f"number of fitted Gaussians {ng} outside 1..{NG_MAX}")
            # src/build_c_g_gauss_STO.F90:6-27 (c_contract = 1, g_contract = zeta)
            if itype == 1:
                c1 = 1.0 * c_fit[ng, 1:ng + 1]
                c2 = np.zeros(ng)
            else:
                c1 = np.zeros(ng)
                c2 = 1.0 * 2.0 * c_fit[ng, 1:ng + 1] * g_fit[ng, 1:ng + 1] * zeta
            gg = zeta * zeta * g_fit[ng, 1:ng + 1]
            for comp in comps:
                suffix = "" if len(comps) == 1 else "_" + "".join(
                    "XYZ"[a] * comp[a] for a in range(3))
                rows.append(dict(center=mol.coords[ia], npower=comp, n_sto=nsto, i_type=itype,
                                 ng=ng, c1=c1, c2=c2, g=gg, zeta=zeta, nucleus=ia,
                                 name=f"{sym}{ia + 1}:{orb}{suffix}", shell=shell_id))
            shell_id += 1
    n = len(rows)
    ld = max([r["ng"] for r in rows] + [1])
    b = Basis(center=np.zeros((n, 3)), npower=np.zeros((n, 3), np.int32),
              n_sto=np.zeros(n, np.int32), i_type=np.zeros(n, np.int32),
              n_gauss=np.zeros(n, np.int32), c_gauss=np.zeros((2, n, ld)),
              g_gauss=np.zeros((n, ld)), g_slater=np.zeros(n), nucleus=np.zeros(n, np.int32),
              names=[], shell=np.zeros(n, np.int32))
    for i, r in enumerate(rows):
        b.center[i] = r["center"]
        b.npower[i] = r["npower"]
        b.n_sto[i] = r["n_sto"]
        b.i_type[i] = r["i_type"]
        b.n_gauss[i] = r["ng"]
        b.c_gauss[0, i, :r["ng"]] = r["c1"]
        b.c_gauss[1, i, :r["ng"]] = r["c2"]
        b.g_gauss[i, :r["ng"]] = r["g"]
        b.g_slater[i] = r["zeta"]
        b.nucleus[i] = r["nucleus"]
        b.names.append(r["name"])
        b.shell[i] = r["shell"]
    return b


def build_mapping(n: int) -> Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Unique quartets (ik|jl), 1-based, in the reference's order
    (src/build_mapping_ijkl.F90:24-43): l outermost, then k, j >= l, i >= k,
    keeping i >= j and dropping i == j with l > k.

    Built one (l, k) block at a time with numpy: inside a block j runs over l..n and, for each
    j, i over max(k, j)..n, skipping i == j when l > k (that i is the first of the run)."""
    npair = n * (n + 1) // 2
    total = npair * (npair + 1) // 2
    out = np.empty((4, total), dtype=np.int32)
    o = 0
    for l in range(1, n + 1):
        js = np.arange(l, n + 1, dtype=np.int64)
        for k in range(1, n + 1):
            start = np.maximum(k, js) + ((l > k) & (js >= k))
            cnt = np.maximum(n - start + 1, 0)
            m = int(cnt.sum())
            if m == 0:
                continue
            jj = np.repeat(js, cnt)
            first = np.repeat(start - np.cumsum(cnt) + cnt, cnt)  # start of each run, shifted
            ii = first + np.arange(m)
            out[0, o:o + m] = ii
            out[1, o:o + m] = jj
            out[2, o:o + m] = k
            out[3, o:o + m] = l
            o += m
    if o != total:
        raise RuntimeError("pb in build_mapping_ijkl")
    return (np.ascontiguousarray(out[0]), np.ascontiguousarray(out[1]),
            np.ascontiguousarray(out[2]), np.ascontiguousarray(out[3]))


def build_mapping_loops(n: int):
    """build_mapping written as the reference's four nested loops (kept as its check)."""
    out = []
    for l in range(1, n + 1):
        for k in range(1, n + 1):
            for j in range(l, n + 1):
                for i in range(k, n + 1):
                    if i == j and l > k:
                        continue
                    if i >= j:
                        out.append((i, j, k, l))
    a = np.array(out, dtype=np.int32).reshape(-1, 4)
    return tuple(np.ascontiguousarray(a[:, c]) for c in range(4))


def count_multi_center(b: "Basis", quartets) -> Dict[int, int]:
    """Number of quartets on 1, 2, 3 and 4 distinct nuclei (count_multi_center_integrals,
    src/count_multi_center_integrals.F90:1-31, with compare_nuclei's ndiff = the number of
    distinct nuclei of (i, j, k, l))."""
    nuc = np.asarray(b.nucleus)
    q = [np.asarray(x) - 1 for x in quartets]
    stacked = np.stack([nuc[q[0]], nuc[q[1]], nuc[q[2]], nuc[q[3]]], axis=1)
    stacked.sort(axis=1)
    ndiff = 1 + (np.diff(stacked, axis=1) != 0).sum(axis=1)
    return {d: int((ndiff == d).sum()) for d in (1, 2, 3, 4)}


def read_j_in(path: str | Path) -> dict:
    """Positional input of two_e_slater (src/two_e_slater.F90:106-154)."""
    L = Path(path).read_text().splitlines()
    it = iter(L)
    next(it)
    num_sim = int(next(it).split()[0])
    next(it)
    molecule = next(it).split()[0]
    next(it)
    basis_file = next(it).split()[0]
    next(it)
    f = next(it).split()
    fit = FitParams(int(f[0]), int(f[1]), int(f[2]), float(f[3].replace("d", "e").replace("D", "e")),
                    int(f[4]))
    next(it)
    npts = int(next(it).split()[0])
    next(it)
    next(it)
    a_zv = float(next(it).split()[0].replace("d", "e").replace("D", "e"))
    if npts % 40 != 0:
        raise ValueError("npts_two_elec must be a multiple of nw")  # src/two_e_slater.F90:148
    return dict(num_simulation=num_sim, molecule=molecule, basis_file=basis_file, fit=fit,
                npts_two_elec=npts, a_zv=a_zv)
