"""The tensor-core primitives of the mixed form (tcgen05 TF32 and FP16 MMA, A in
Tensor Memory, B in shared memory in the canonical no-swizzle layout, FP32
accumulator in Tensor Memory): exact integer products pin the operand and
accumulator layouts; random operands match a TF32-rounded FP64 product."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tc(A, B):
    from periodsearch_gb300 import _abi

    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    D = np.zeros((128, 32), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))   # noqa: E731
    _abi.check(_abi.lib().ps_tc_selftest(0, fp(A), fp(B), A.shape[1], fp(D)), "ps_tc_selftest")
    return D


def _tf32(x):
    """Round to TF32 (10 explicit mantissa bits), nearest, ties away from zero."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x1000) & 0xFFFFE000
    return b.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("K", [8, 288, 480])
def test_tc_integer_products_exact(engine_lib, K):
    rng = np.random.default_rng(K)
    A = rng.integers(-8, 9, (128, K)).astype(np.float32)
    B = rng.integers(-8, 9, (32, K)).astype(np.float32)
    np.testing.assert_array_equal(_tc(A, B), A.astype(np.float64) @ B.T.astype(np.float64))


def test_tc_rows_and_columns_land_in_place(engine_lib):
    """One-hot operands: D[m][n] = A[m][k] B[n][k] for a single k, so every
    element of D identifies its row and column."""
    K = 64
    A = np.zeros((128, K), np.float32)
    B = np.zeros((32, K), np.float32)
    A[:, 5] = np.arange(128) + 1
    B[:, 5] = 256 * (np.arange(32) + 1)        # exact in TF32 (11 significant bits)
    D = _tc(A, B)
    np.testing.assert_array_equal(D, np.outer(np.arange(128) + 1, 256 * (np.arange(32) + 1)))


def test_tc_random_matches_tf32_reference(engine_lib):
    rng = np.random.default_rng(7)
    A = rng.normal(size=(128, 288)).astype(np.float32)
    B = rng.normal(size=(32, 288)).astype(np.float32)
    ref = _tf32(A).astype(np.float64) @ _tf32(B).T.astype(np.float64)
    got = _tc(A, B)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).T.astype(np.float64)
    assert np.max(np.abs(got - ref) / scale) < 1e-5


def _tc16(A, B):
    from periodsearch_gb300 import _abi

    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    D = np.zeros((128, 32), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))   # noqa: E731
    _abi.check(_abi.lib().ps_tc_selftest_f16(0, fp(A), fp(B), A.shape[1], fp(D)), "ps_tc_selftest_f16")
    return D


@pytest.mark.parametrize("K", [16, 288, 512])
def test_tc_f16_integer_products_exact(engine_lib, K):
    """FP16 operands (two per Tensor Memory column, K = 16 per MMA)."""
    rng = np.random.default_rng(100 + K)
    A = rng.integers(-8, 9, (128, K)).astype(np.float32)
    B = rng.integers(-8, 9, (32, K)).astype(np.float32)
    np.testing.assert_array_equal(_tc16(A, B), A.astype(np.float64) @ B.T.astype(np.float64))


@pytest.mark.parametrize("k", [4, 5, 14, 15, 33])
def test_tc_f16_pairs_packed_in_k_order(engine_lib, k):
    """One-hot operands at an even and an odd K index: the two FP16 halves
    of a column and the K order of the core matrices land in place."""
    K = 48
    A = np.zeros((128, K), np.float32)
    B = np.zeros((32, K), np.float32)
    A[:, k] = np.arange(128) + 1
    B[:, k] = 8 * (np.arange(32) + 1)          # exact in FP16
    A[:, k ^ 1] = 1000                          # the other half of the pair: must meet zeros in B
    D = _tc16(A, B)
    np.testing.assert_array_equal(D, np.outer(np.arange(128) + 1, 8 * (np.arange(32) + 1)))


def test_tc_f16_random_matches_f16_reference(engine_lib):
    rng = np.random.default_rng(9)
    A = rng.normal(size=(128, 288)).astype(np.float32)
    B = rng.normal(size=(32, 288)).astype(np.float32)
    ref = A.astype(np.float16).astype(np.float64) @ B.astype(np.float16).T.astype(np.float64)
    got = _tc16(A, B)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).T.astype(np.float64)
    assert np.max(np.abs(got - ref) / scale) < 1e-5


def test_bounded_wait_gives_up_and_context_stays_usable(engine_lib):
    """A wait on an mbarrier phase that nothing completes gives up after its
    poll limit, reports PS_ERR_TIMEOUT and frees its Tensor Memory; the
    device context then still runs the tensor-core self-test (exact integer
    products) and a mixed-form scan that matches the FP64 form."""
    from conftest import GOLDEN
    from periodsearch_gb300 import PS_FORM_FP64, PS_FORM_MIXED, Engine, _abi, read_input

    L = _abi.lib()
    assert L.ps_tc_wait_selftest(0, 64) == _abi.PS_ERR_TIMEOUT
    assert L.ps_tc_wait_selftest(0, 0) == _abi.PS_ERR_ARG
    assert L.ps_tc_wait_selftest(0, 4096) == _abi.PS_ERR_TIMEOUT     # twice in a row
    rng = np.random.default_rng(11)
    A = rng.integers(-8, 9, (128, 64)).astype(np.float32)
    B = rng.integers(-8, 9, (32, 64)).astype(np.float32)
    np.testing.assert_array_equal(_tc(A, B), A.astype(np.float64) @ B.T.astype(np.float64))
    data = read_input(GOLDEN / "tiny_cal" / "period_search_in")
    with Engine(data, form=PS_FORM_MIXED) as eng, Engine(data, form=PS_FORM_FP64) as e64:
        assert eng.info.tensor_cores == 1
        conw_r = eng.info.conw_r0
        mixed = eng.scan(conw_r, 1, 3)
        ref = e64.scan(conw_r, 1, 3)
    np.testing.assert_allclose(mixed["rms"], ref["rms"], rtol=5e-2)
