"""Interpolative decomposition of the host set-up (pivoted QR and skeleton
rows, H2P-ERI src/H2E_ID_compress.c:51-184 and :491-576) against LAPACK's
column-pivoted QR (scipy.linalg.qr with pivoting: xGEQP3 takes the same
greedy pivot, the remaining column of largest norm). The set-up's QR is
blocked (pending updates of up to 32 reflectors) and recomputes a column norm
only where the downdated one has lost its accuracy, so these tests pin that
it still picks the reference's pivots and stops at the reference's rank."""
import ctypes

import numpy as np
import pytest

sla = pytest.importorskip("scipy.linalg")


@pytest.fixture(scope="module")
def L(library):
    library.h2g_id_rows.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                    ctypes.c_void_p, ctypes.c_void_p]
    library.h2g_id_rows.restype = ctypes.c_int
    return library


def id_rows(L, A, tol):
    nrow, ncol = A.shape
    A = np.ascontiguousarray(A, dtype=np.float64)
    J = np.zeros(max(nrow, 1), dtype=np.int32)
    U = np.zeros(max(nrow * min(nrow, ncol), 1))
    r = L.h2g_id_rows(nrow, ncol, A.ctypes.data, tol, J.ctypes.data, U.ctypes.data)
    return r, J[:r].copy(), U[:nrow * r].reshape(nrow, r)


def graded(rng, nrow, ncol, k, decay):
    """nrow x ncol matrix of rank k with singular values decay**i."""
    Q1, _ = np.linalg.qr(rng.standard_normal((nrow, k)))
    Q2, _ = np.linalg.qr(rng.standard_normal((ncol, k)))
    return (Q1 * decay ** np.arange(k)) @ Q2.T


def lapack_rank_and_pivots(A, tol):
    """Rank by the reference's stopping rule on LAPACK's pivoted QR of A^T."""
    m = A.shape[1]
    _, R, P = sla.qr(A.T, mode="economic", pivoting=True)
    norm0 = np.linalg.norm(A, axis=1).max()
    stop = max(np.sqrt(m) * 1e-15, tol) * norm0
    d = np.abs(np.diag(R))
    r = int(np.argmax(d < stop)) if (d < stop).any() else len(d)
    return r, P


@pytest.mark.parametrize("nrow,ncol,k,decay,tol", [
    (300, 600, 120, 0.82, 1e-8),     # the U-construction shape (2x as many sketch columns as rows)
    (250, 180, 150, 0.85, 1e-6),     # more rows than columns (a near-field D block)
    (97, 61, 40, 0.6, 1e-6),         # odd sizes, rank reached inside the first block
])
def test_id_matches_lapack_pivoting(L, nrow, ncol, k, decay, tol):
    rng = np.random.default_rng(nrow * 1000 + ncol)
    A = graded(rng, nrow, ncol, k, decay)
    r, J, U = id_rows(L, A, tol)
    r_ref, P = lapack_rank_and_pivots(A, tol)
    assert abs(r - r_ref) <= 1
    assert len(set(J) & set(P[:r_ref])) >= min(r, r_ref) - 2
    assert np.all(np.diff(J) > 0)                        # sorted skeleton rows
    np.testing.assert_array_equal(U[J], np.eye(r))      # skeleton rows reproduce themselves
    err = np.linalg.norm(A - U @ A[J]) / np.linalg.norm(A)
    assert err < 5 * tol


def test_id_exact_low_rank_and_zero(L):
    rng = np.random.default_rng(5)
    A = graded(rng, 64, 128, 7, 1.0)                     # exact rank 7
    r, J, U = id_rows(L, A, 1e-10)
    assert r == 7
    assert np.linalg.norm(A - U @ A[J]) < 1e-12 * np.linalg.norm(A)
    r0, J0, _ = id_rows(L, np.zeros((10, 20)), 1e-8)     # a zero block has rank 0
    assert r0 == 0 and len(J0) == 0


def test_id_rows_in_the_span_of_others(L):
    """Exact rank with rows that are combinations of other rows (they fall
    below the stop norm as the span fills and leave the per-step work) and
    rows that are negligible from the start: the rank is the span's, and the
    coefficients of every non-skeleton row reproduce it."""
    rng = np.random.default_rng(21)
    B = graded(rng, 40, 260, 40, 0.8)                     # 40 independent rows, graded
    M = rng.standard_normal((70, 40)) * 0.3
    tiny = 1e-14 * rng.standard_normal((20, 260))
    A = np.vstack([B, M @ B, tiny])[rng.permutation(130)]
    r, J, U = id_rows(L, A, 1e-10)
    assert r == 40
    assert np.linalg.norm(A - U @ A[J]) < 1e-9 * np.linalg.norm(A)
    r_ref, P = lapack_rank_and_pivots(A, 1e-10)
    assert r_ref == 40 and len(set(J) & set(P[:r_ref])) >= 38
