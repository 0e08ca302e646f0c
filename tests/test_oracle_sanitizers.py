"""The CPU oracle built with AddressSanitizer and UndefinedBehaviorSanitizer runs its analytic,
one-centre, one-electron and faithful ZV-MC paths on the minimal H2O basis without a report
(the oracle is C; this is its memory-safety check)."""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from slater_stoch_gb300 import basis, configs
from oracle import binding as O
b = configs.h2o_minimal(ng0=4); q = basis.build_mapping(b.n); ob = O.OracleBasis(b)
pre = O.precond(ob); g, _ = O.gauss_eri(ob, q, pre)
O.set_sum_mode("extended"); g2, _ = O.gauss_eri(ob, q, pre)
v, m = O.monocenter(ob, q)
S, V, K = O.one_elect(ob, [[0, 0, 0], [0, 1.4305, 1.1093], [0, -1.4305, 1.1093]], [8.0, 1.0, 1.0])
rng = np.random.default_rng(0)
r1 = rng.standard_normal((400, 3)); r2 = rng.standard_normal((400, 3))
O.zvmc_faithful(ob, q, 1.8, r1, r2, nblocks=2, npts=200)
print("sanitized run ok", int(m.sum()))
"""


def test_oracle_under_asan_ubsan(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    asan = subprocess.run([gcc, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not asan or not Path(asan).exists():
        pytest.skip("libasan not available")
    lib = tmp_path / "libss_oracle_san.so"
    subprocess.run([gcc, "-O1", "-g", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                    "-D_GNU_SOURCE", "-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-o", str(lib),
                    str(ROOT / "oracle" / "ss_oracle.c"), "-lm"], check=True)
    env = dict(os.environ, SS_ORACLE_LIB=str(lib), LD_PRELOAD=asan,
               ASAN_OPTIONS="detect_leaks=0:halt_on_error=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "sanitized run ok" in r.stdout
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr
