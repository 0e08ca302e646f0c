"""tcgen05 split-BF16 contraction (the shared estimator's GEMM) vs an FP64 numpy product.

Shapes cover one partial tile (P < 128), exact tiles, ragged multi-tile P (all four epilogue
warps and all 32-column TMEM chunks), K slices longer than the 3-stage shared-memory ring, and
explicit / automatic K splits.  Gate: |C - C_ref| <= 2e-6 * sum_k |a_k b_k| (FP32 accumulation).
"""
import numpy as np
import pytest

from slater_stoch_gb300 import api

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def bits_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def split(x):
    hi = bf16_bits(x)
    lo = bf16_bits(x.astype(np.float32) - bits_to_f64(hi).astype(np.float32))
    return hi, lo


@pytest.mark.parametrize("P,K,ksplit", [(28, 64, 1), (128, 128, 1), (130, 256, 2), (200, 64 * 7, 1),
                                        (351, 8192, 0), (257, 64 * 9, 3)])
def test_split_bf16_gemm(P, K, ksplit):
    rng = np.random.default_rng(P * 1000 + K)
    A = rng.standard_normal((P, K)).astype(np.float32) * np.exp(rng.uniform(-3, 3, (P, 1))).astype(np.float32)
    B = rng.standard_normal((P, K)).astype(np.float32)
    ah, al = split(A)
    bh, bl = split(B)
    Ah, Al, Bh, Bl = (bits_to_f64(t) for t in (ah, al, bh, bl))
    ref = Ah @ Bh.T + Ah @ Bl.T + Al @ Bh.T
    mag = np.abs(Ah) @ np.abs(Bh).T
    with api.Context(0) as ctx:
        C = ctx.split_bf16_gemm(ah, al, bh, bl, ksplit=ksplit)
    err = np.abs(C - ref)
    bad = np.argwhere(err > 2e-6 * mag + 1e-30)
    assert bad.size == 0, f"{len(bad)} bad entries, first {bad[:5].tolist()}, max rel {np.max(err / mag):.3g}"
    # the split keeps ~16 bits: against the unsplit FP32 product the error is ~2^-16 relative
    full = A.astype(np.float64) @ B.astype(np.float64).T
    assert np.max(np.abs(C - full) / (np.abs(A).astype(np.float64) @ np.abs(B).T)) < 1e-4
