"""Tensor-core (tcgen05, TF32) GEMM self-test against a host FP64 product.

Shapes with K >= 1024 run split along K (partials + ordered reduction).
Error is measured relative to sum_k |a_ik b_kj| (+ |beta c_ij|) per entry:
plain TF32 rounds each operand to 11 significant bits (bound 2^-10 per
product, so 2e-3 with margin); split TF32 keeps the A_lo B_lo term out only
(FP32 accumulation dominates: 1e-5); split BF16 (split = 2, the schur_bf16
products: hi = bf16(a), lo = bf16(a - hi), three kind::f16 MMAs) carries 16
significant bits per operand and drops lo x lo (2^-16 each: 1e-4).
"""
import ctypes

import pytest

import rank_structured_cholesky_gb300 as rs

pytestmark = pytest.mark.gpu

SHAPES = [
    (128, 64, 32, 0, 0), (100, 50, 7, 0, 1), (300, 130, 257, 1, 0), (257, 200, 96, 1, 1),
    (64, 300, 1000, 0, 0), (1000, 64, 64, 0, 1), (5, 3, 1, 0, 0),
    # A plain and B transposed with K a multiple of 4: the cp.async path (ragged M, N and K tails)
    (200, 130, 96, 0, 1), (130, 70, 36, 0, 1), (64, 64, 44, 0, 1), (257, 129, 500, 0, 1),
    # K >= 1024: four K slices summed by the split-K reduction
    (300, 104, 2048, 1, 0), (129, 65, 3001, 0, 1), (129, 65, 3000, 0, 1),
    # 128-wide tiles (N > 64) with either operand layout; unaligned leading
    # dimensions (no 16-byte loads); the sketch shapes of the factor
    (300, 128, 64, 0, 0), (333, 100, 37, 1, 1), (250, 127, 130, 1, 0), (3072, 69, 1024, 1, 0),
    (1024, 104, 3000, 0, 0), (512, 129, 45, 0, 1),
]


TOL = {0: 2e-3, 1: 1e-5, 2: 1e-4}


@pytest.mark.parametrize("split", [0, 1, 2])
@pytest.mark.parametrize("shape", SHAPES)
def test_tensor_core_gemm(shape, split):
    M, N, K, tA, tB = shape
    out = (ctypes.c_double * 3)()
    st = rs.load_library().rschol_selftest_gemm(M, N, K, tA, tB, split, 0, out)
    assert st == 0, st
    assert out[0] < TOL[split], (shape, split, out[0], out[1])
    # A and B K-major with 16-byte rows (K a multiple of 4) in a TF32 launch: TMA staging
    assert out[2] == (1.0 if (tA == 0 and tB == 1 and K % 4 == 0 and split != 2) else 0.0), out[2]


@pytest.mark.parametrize("split", [1, 2])
@pytest.mark.parametrize("n", [60, 400])
def test_tensor_core_gemm_lower_tiles(n, split):
    # n = 400: 128-wide tiles, those strictly above the diagonal skipped
    out = (ctypes.c_double * 3)()
    st = rs.load_library().rschol_selftest_gemm(n, n, 64, 0, 1, split, 1, out)
    assert st == 0 and out[0] < TOL[split], (st, out[0])


@pytest.mark.parametrize("split", [0, 1, 2])
def test_bench_gemm_times_a_launch(split):
    ms = ctypes.c_double()
    st = rs.load_library().rschol_bench_gemm(1024, 256, 512, split, 3, ctypes.byref(ms))
    assert st == 0 and 0 < ms.value < 1e3, (st, ms.value)
