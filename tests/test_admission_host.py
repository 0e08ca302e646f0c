"""Admission of asynchronous jobs (csrc/admission.h) on the host with fake jobs: submission
order, the concurrency limit, the footprint budget, refusal of a job larger than the budget,
abandoned tickets, and no stranded job when a single job exceeds what is left."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "slater_stoch_gb300" / "csrc"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("adm") / "libadm_host.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread", "-shared", "-fPIC", f"-I{CSRC}",
                    str(HERE / "admission_host_shim.cpp"), "-o", str(out)], check=True)
    L = C.CDLL(str(out))
    i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
    L.ss_host_admission_run.argtypes = [C.c_int, i64p, i32p, C.c_longlong, C.c_int, C.c_int, i32p, i32p,
                                        C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                                        C.POINTER(C.c_longlong)]
    return L


def _run(lib, bytes_, budget=0, max_running=0, abandon=None, sleep_ms=15):
    n = len(bytes_)
    b = np.ascontiguousarray(bytes_, np.int64)
    ab = np.zeros(n, np.int32) if abandon is None else np.ascontiguousarray(abandon, np.int32)
    order = np.zeros(n, np.int32)
    refused = np.zeros(n, np.int32)
    pr, pb, spr, spb = C.c_int(), C.c_longlong(), C.c_int(), C.c_longlong()
    rc = lib.ss_host_admission_run(n, b, ab, budget, max_running, sleep_ms, order, refused, C.byref(pr),
                                   C.byref(pb), C.byref(spr), C.byref(spb))
    assert rc == 0  # nothing left running or queued
    return order, refused.astype(bool), pr.value, pb.value, spr.value, spb.value


def test_concurrency_limit_and_fifo(lib):
    order, refused, pr, pb, spr, spb = _run(lib, [100] * 6, max_running=2, sleep_ms=50)
    assert not refused.any() and 1 <= pr <= 2 and 1 <= spr <= 2
    assert list(order) == list(range(6))  # started in submission order


def test_budget_limits_the_summed_footprint(lib):
    order, refused, pr, pb, spr, spb = _run(lib, [100] * 6, budget=250)
    assert pb <= 250 and spb <= 250 and pr <= 2
    assert sorted(order) == list(range(6))


def test_job_larger_than_budget_is_refused(lib):
    order, refused, *_ = _run(lib, [100, 300, 100], budget=250)
    assert list(refused) == [False, True, False] and order[1] == -1
    assert order[0] == 0 and order[2] == 1


def test_abandoned_ticket_does_not_block_the_queue(lib):
    order, refused, pr, *_ = _run(lib, [100] * 4, max_running=1, abandon=[0, 1, 0, 0])
    assert order[1] == -1 and sorted(order[[0, 2, 3]]) == [0, 1, 2]


def test_unlimited_runs_all_at_once(lib):
    order, refused, pr, pb, spr, spb = _run(lib, [100] * 4, sleep_ms=1000)
    assert spr >= 2 and spb == 100 * spr  # jobs overlap when nothing limits them


def test_admission_under_thread_sanitizer(tmp_path):
    """The admission scenarios built as a standalone program with ThreadSanitizer: no data race
    is reported and every queue drains."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "adm_tsan"
    r = subprocess.run([gxx, "-O1", "-g", "-std=c++17", "-pthread", "-fsanitize=thread", "-DSS_ADMISSION_MAIN",
                        f"-I{CSRC}", str(HERE / "admission_host_shim.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("ThreadSanitizer build not available: " + r.stderr[-200:])
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300,
                         env={"TSAN_OPTIONS": "halt_on_error=1"})
    assert "ThreadSanitizer" not in run.stderr, run.stderr[-3000:]
    assert run.returncode == 0
