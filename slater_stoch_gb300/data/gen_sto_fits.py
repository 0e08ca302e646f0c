"""Regenerate ``sto_fits.txt``: the STO -> n-Gaussian fit tables.

The two-electron path fits every Slater-type orbital exp(-r) by
``sum_m c_m exp(-g_m r^2)`` with tabulated (c, g) for n = 1..30 Gaussians
(the "SMILES" fits, ``src/read_fit_SMILES.F90:1-1399`` of the reference,
``c_fit_exp(m, n)`` / ``g_fit_exp(m, n)``).  The numbers are data that must
be identical to the reference's for the Gaussian-fit ERIs to agree, so this
script extracts them verbatim into a plain text table

    n  m  c_fit  g_fit

one row per (n, m), m = 1..n.  Run it where a checkout of the reference exists:

    python gen_sto_fits.py <path of the reference checkout>

The generated file is committed; nothing reads the reference at run time.
"""
import re
import sys
from pathlib import Path


def main(ref_root: str) -> None:
    src = Path(ref_root) / "src" / "read_fit_SMILES.F90"
    text = src.read_text()
    pat = re.compile(r"([cg])_fit_exp\(\s*(\d+)\s*,\s*(\d+)\s*\)\s*=\s*([-+0-9.DdEe]+)")
    table = {}
    for kind, m, n, val in pat.findall(text):
        v = float(val.replace("D", "e").replace("d", "e"))
        table.setdefault((int(n), int(m)), {})[kind] = v
    out = Path(__file__).with_name("sto_fits.txt")
    rows = []
    for (n, m) in sorted(table):
        e = table[(n, m)]
        rows.append(f"{n:3d} {m:3d} {e['c']!r} {e['g']!r}")
    # every n = 1..30 must be complete
    for n in range(1, 31):
        for m in range(1, n + 1):
            assert (n, m) in table and len(table[(n, m)]) == 2, (n, m)
    out.write_text("# n m c_fit g_fit  (STO exp(-r) ~ sum_m c exp(-g r^2))\n" + "\n".join(rows) + "\n")
    print(f"wrote {out} ({len(rows)} rows)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python gen_sto_fits.py <path of the reference checkout>")
    main(sys.argv[1])
