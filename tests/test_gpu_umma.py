"""The tensor-core (tcgen05) operand layouts of the multi-density kernel,
checked against exact integer arithmetic: one 128 x 128 tile of integers
(bf16-exact) times 16 vectors on both sides, N = A X^T with A K-major and
T = A^T Y^T with the same shared-memory bytes read MN-major. The FP32
accumulation of integer products must be exact while every partial sum stays
below 2^24, which the multi-density kernel's slice scheme relies on."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(library, A, X, Y):
    fn = library.h2g_selftest_umma
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 5
    A, X, Y = (np.ascontiguousarray(a, dtype=np.float32) for a in (A, X, Y))
    N = np.zeros((128, 16), np.float32)
    T = np.zeros((128, 16), np.float32)
    rc = fn(A.ctypes.data, X.ctypes.data, Y.ctypes.data, N.ctypes.data, T.ctypes.data)
    assert rc == 0, library.H2ERI_gpu_last_error()
    return N.astype(np.int64), T.astype(np.int64)


def test_umma_layouts_exact(library):
    rng = np.random.default_rng(11)
    A = rng.integers(-128, 129, size=(128, 128))
    X = rng.integers(-128, 129, size=(16, 128))
    Y = rng.integers(-128, 129, size=(16, 128))
    eN, eT = A @ X.T, A.T @ Y.T
    N, T = _run(library, A, X, Y)
    np.testing.assert_array_equal(N, eN)
    np.testing.assert_array_equal(T, eT)


def test_umma_integer_sums_near_2_to_24_are_exact(library):
    """Largest partial sums of the slice scheme: 128 products of 256 x 255
    (8.4e6 < 2^24), with a row of mixed signs."""
    A = np.full((128, 128), 256)
    X = np.full((16, 128), 255)
    Y = np.full((16, 128), -255)
    A[5, ::2] = -256
    X[3, ::3] = 1
    eN, eT = A @ X.T, A.T @ Y.T
    assert np.abs(eN).max() < 2 ** 24 and np.abs(eT).max() < 2 ** 24
    N, T = _run(library, A, X, Y)
    np.testing.assert_array_equal(N, eN)
    np.testing.assert_array_equal(T, eT)
