"""The tcgen05 tensor-core GEMM (bem_tc_gemm_f32) against an FP64 numpy
product of the same FP32 inputs.

Error measures: entry-wise, max over outputs of |C - C_ref| / (|A| |B|)_entry
(the bound a product of FP32 data can be held to), on data spanning two
decades per operand (wider than the solver's operands); norm-wise,
||C - C_ref||_F / (||A||_F ||B||_F), on data spanning six decades per
operand.  The operands are scaled by a power of two per matrix (A) and per
column (B) and split into fp16 parts, so entries far below their operand's
largest keep an absolute, not a relative, precision of 2^-24 of it (fp16
subnormals): entry-wise bounds then hold only relative to the largest
products, which the norm-wise measure states.  The tensor core adds the
products into its FP32 accumulator without IEEE round-to-nearest (errors grow
like sqrt(K) 2^-24, several times numpy's blocked FP32 sums), so the
entry-wise tolerance is 4 sqrt(K) 2^-24 (+ 2^-21 for the two-part split's
dropped term), under the worst-case FP32 bound K 2^-24; norm-wise 1e-6
(parts = 2) and 1e-7 (parts = 3).  The shapes
cover both operand orders, ragged M/K/N (every tile edge), the four N-tile
widths and split-K (few output tiles over a long K)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _err(C, A, B, trans):
    opA = (A.T if trans else A).astype(np.float64)
    ref = opA @ B.astype(np.float64)
    scale = np.abs(opA) @ np.abs(B.astype(np.float64))
    return float(np.max(np.abs(C.astype(np.float64) - ref) / np.maximum(scale, 1e-300)))


def _data(rng, shape, decades=2.0):
    return (rng.standard_normal(shape) * 10.0 ** rng.uniform(-decades / 2, decades / 2, shape)).astype(np.float32)


def _err_norm(C, A, B, trans):
    opA = (A.T if trans else A).astype(np.float64)
    ref = opA @ B.astype(np.float64)
    return float(np.linalg.norm(C.astype(np.float64) - ref) / (np.linalg.norm(opA) * np.linalg.norm(B)))


@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("m,k,n", [(300, 517, 37), (1000, 777, 130), (129, 64, 256), (256, 8192, 32),
                                   (77, 1500, 300), (1, 5, 1)])
@pytest.mark.parametrize("parts", [2, 3])
def test_tc_gemm_matches_fp64(bemlib, trans, m, k, n, parts):
    rng = np.random.default_rng(m * 7 + k * 3 + n + parts)
    A = _data(rng, (k, m) if trans else (m, k))
    B = _data(rng, (k, n))
    C = bemlib.tc_gemm(A, B, trans=trans, parts=parts)
    err = _err(C, A, B, trans)
    tol = 4 * np.sqrt(k) * 2.0 ** -24 + (2.0 ** -21 if parts == 2 else 0.0)
    assert err < tol, (err, tol)


@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("parts,tol", [(2, 1e-6), (3, 1e-7)])
def test_tc_gemm_wide_range_normwise(bemlib, trans, parts, tol):
    rng = np.random.default_rng(11 + parts)
    m, k, n = 300, 517, 37
    A = _data(rng, (k, m) if trans else (m, k), decades=6.0)
    B = _data(rng, (k, n), decades=6.0)
    C = bemlib.tc_gemm(A, B, trans=trans, parts=parts)
    assert _err_norm(C, A, B, trans) < tol


def test_tc_gemm_repeatable(bemlib):
    """Same inputs, same bits (fixed accumulation order, split-K partial sums
    added in fixed order)."""
    rng = np.random.default_rng(5)
    A = _data(rng, (256, 8192))
    B = _data(rng, (8192, 32))
    C1 = bemlib.tc_gemm(A, B, parts=2)
    C2 = bemlib.tc_gemm(A, B, parts=2)
    assert np.array_equal(C1, C2)


def test_tc_gemm_rejects_bad_parts(bemlib):
    with pytest.raises(bemlib.BemError):
        bemlib.tc_gemm(np.ones((4, 4), np.float32), np.ones((4, 4), np.float32), parts=4)
