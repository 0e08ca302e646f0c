"""Regenerate the committed oracle fixtures under tests/golden/.

The fixtures hold outputs of the CPU oracle (oracle/ss_oracle.c, a restatement of the
reference's algorithms) at sizes too slow to recompute in every test run:
  gauss_eri_h2o_minimal_ng20.npz : all 406 (ik|jl) of the 7-function H2O basis with
                                   20-Gaussian fits, plus the Schwarz diagonal; `eri` is the
                                   reference's sequential FP64 sum, `eri_ext` the same terms
                                   accumulated in long double.
Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import binding as O  # noqa: E402
from slater_stoch_gb300 import basis, configs  # noqa: E402


def main():
    out = Path(__file__).parent
    b = configs.h2o_minimal(ng0=20)
    q = basis.build_mapping(b.n)
    ob = O.OracleBasis(b)
    O.set_sum_mode("extended")
    pre = O.precond(ob)
    eri_ext, nz = O.gauss_eri(ob, q, pre)
    O.set_sum_mode("reference")
    eri, _ = O.gauss_eri(ob, q, pre)
    np.savez_compressed(out / "gauss_eri_h2o_minimal_ng20.npz", eri=eri, eri_ext=eri_ext,
                        precond=pre, n_removed=np.array(nz))
    print("wrote", out / "gauss_eri_h2o_minimal_ng20.npz")


if __name__ == "__main__":
    main()
