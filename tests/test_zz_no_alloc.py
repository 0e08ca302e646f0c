"""The allocation-free contraction entry point (ss_split_bf16_gemm_noalloc).

Some callers cannot allocate device memory: their device memory belongs to their own pool, or
they run where cudaMalloc is not allowed.  The entry point takes the caller's device buffers
and keeps its K-slice partial products in a fixed array inside the library.  This test calls
it through the C ABI on buffers the test allocates, twice in a row with different data, and
checks each result against the FP64 product of the same BF16 hi/lo operands (numpy) and
against the allocating entry point (ss_split_bf16_gemm), within the tolerance of the
contraction's own test: |C - C_ref| <= 2e-6 * sum_k |a_k b_k| (FP32 accumulation).  The largest
size the fixed array takes (P = 2048, where the partials of one K slice fill it and a requested
split of 8 is cut to 1) is run the same way.  Sizes beyond the fixed array are rejected before
anything runs.  The file is named so that pytest collects it last.
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


def _run(L, ctx, P, K, ksplit, seed, scale):
    import torch
    rng = np.random.default_rng(seed)
    A = (rng.standard_normal((P, K)) * np.exp(rng.uniform(-2, 2, (P, 1)))).astype(np.float32)
    B = (rng.standard_normal((P, K)) * scale).astype(np.float32)
    ah, al = _split(A)
    bh, bl = _split(B)
    Ah, Al, Bh, Bl = (_as_f64(t) for t in (ah, al, bh, bl))
    exact = Ah @ Bh.T + Ah @ Bl.T + Al @ Bh.T          # FP64 product of the same operands
    mag = np.abs(Ah) @ np.abs(Bh).T
    alloc = ctx.split_bf16_gemm(ah, al, bh, bl, ksplit=ksplit)
    stream = torch.cuda.current_stream()
    dev = [torch.from_numpy(t.view(np.int16)).to("cuda") for t in (ah, al, bh, bl)]
    d_c = torch.full((P, P), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = L.ss_split_bf16_gemm_noalloc(C.c_void_p(stream.cuda_stream), P, K,
                                      *[C.c_void_p(t.data_ptr()) for t in dev], ksplit,
                                      C.c_void_p(d_c.data_ptr()))
    _lib.check(rc)
    got = d_c.cpu().numpy()
    assert np.all(np.isfinite(got))
    for ref, what in ((exact, "FP64 product"), (alloc, "ss_split_bf16_gemm")):
        err = np.abs(got - ref)
        assert np.all(err <= 2e-6 * mag + 1e-30), f"vs {what}: max rel {np.max(err / mag):.3g}"


def test_noalloc_matches_fp64_and_allocating_entry_point():
    """Two calls in a row with different data (the second must not see the first's partials)."""
    L = _lib.load()
    with api.Context(0) as ctx:
        for trial in range(2):
            _run(L, ctx, 351, 64 * 130, 0, 100 + trial, 1 + trial)


def test_noalloc_largest_size():
    """P = 2048 fills the fixed array with one K slice: the requested split of 8 is cut to 1."""
    L = _lib.load()
    with api.Context(0) as ctx:
        for trial in range(2):
            _run(L, ctx, 2048, 128, 8, 200 + trial, 1 + trial)


def test_noalloc_rejects_oversize():
    L = _lib.load()
    z = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ss_split_bf16_gemm_noalloc(None, 2049, 64, z, z, z, z, 0, z)
    assert rc == -1 and b"P <= 2048" in L.ss_last_error()
