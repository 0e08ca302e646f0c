"""The allocation-free contraction entry point (ss_split_bf16_gemm_noalloc).

Some callers cannot allocate device memory: their device memory belongs to their own pool, or
they run where cudaMalloc is not allowed.  The entry point takes the caller's device buffers
and keeps its K-slice partial products in a fixed array inside the library.  This test calls
it through the C ABI on buffers the test allocates, twice in a row with different data, and
checks each result against the allocating entry point (ss_split_bf16_gemm) on the same
operands, within the tolerance of the contraction's own test.  It also checks that sizes
beyond the fixed array are rejected before anything runs.  The file is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from slater_stoch_gb300 import _lib, api

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _as_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def _split(x):
    hi = _bf16_bits(x)
    lo = _bf16_bits(x.astype(np.float32) - _as_f64(hi).astype(np.float32))
    return hi, lo


def test_noalloc_matches_allocating_entry_point():
    import torch
    L = _lib.load()
    P, K = 351, 64 * 130
    stream = torch.cuda.current_stream()
    with api.Context(0) as ctx:
        for trial in range(2):
            rng = np.random.default_rng(100 + trial)
            A = rng.standard_normal((P, K)).astype(np.float32)
            B = (rng.standard_normal((P, K)) * (1 + trial)).astype(np.float32)
            ah, al = _split(A)
            bh, bl = _split(B)
            ref = ctx.split_bf16_gemm(ah, al, bh, bl, ksplit=0)
            dev = [torch.from_numpy(t.view(np.int16)).to("cuda") for t in (ah, al, bh, bl)]
            d_c = torch.full((P, P), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            rc = L.ss_split_bf16_gemm_noalloc(C.c_void_p(stream.cuda_stream), P, K,
                                              *[C.c_void_p(t.data_ptr()) for t in dev], 0,
                                              C.c_void_p(d_c.data_ptr()))
            _lib.check(rc)
            got = d_c.cpu().numpy()
            mag = np.abs(_as_f64(ah)) @ np.abs(_as_f64(bh)).T
            assert np.all(np.isfinite(got))
            assert np.all(np.abs(got - ref) <= 2e-6 * mag + 1e-30), np.max(np.abs(got - ref) / mag)


def test_noalloc_rejects_oversize():
    L = _lib.load()
    z = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ss_split_bf16_gemm_noalloc(None, 2049, 64, z, z, z, z, 0, z)
    assert rc == -1 and b"P <= 2048" in L.ss_last_error()
