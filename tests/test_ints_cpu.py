"""Integral engine (host, feeds the set-up): Boys function against
arbitrary-precision values and ERI permutational symmetry."""
import ctypes

import numpy as np
import pytest

import h2eri_gb300 as hg


class Shell(ctypes.Structure):
    _fields_ = [("am", ctypes.c_int), ("nprim", ctypes.c_int), ("x", ctypes.c_double), ("y", ctypes.c_double),
                ("z", ctypes.c_double), ("alpha", ctypes.POINTER(ctypes.c_double)),
                ("coef", ctypes.POINTER(ctypes.c_double))]


class Pair(ctypes.Structure):
    _fields_ = [("am1", ctypes.c_int), ("am2", ctypes.c_int), ("nprim", ctypes.c_int),
                ("A", ctypes.c_double * 3), ("B", ctypes.c_double * 3)] + \
               [(n, ctypes.POINTER(ctypes.c_double)) for n in ("P", "p", "K", "ip")]


def ncart(l):
    return (l + 1) * (l + 2) // 2


@pytest.fixture(scope="module")
def L(library):
    library.h2g_ints_init()
    library.h2g_boys.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    library.h2g_pair_init.argtypes = [ctypes.POINTER(Pair), ctypes.POINTER(Shell), ctypes.POINTER(Shell)]
    library.h2g_eri_quartet.argtypes = [ctypes.POINTER(Pair), ctypes.POINTER(Pair), ctypes.c_void_p]
    library.h2g_normalize_shell.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return library


def test_boys_against_mpmath(L):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    out = np.zeros(17)
    for T in (0.0, 1e-9, 0.013, 0.5, 1.7, 7.3, 19.99, 33.3, 39.99, 40.0, 55.0, 120.0):
        L.h2g_boys(16, T, out.ctypes.data)
        for m in range(17):
            if T == 0.0:
                ref = mp.mpf(1) / (2 * m + 1)
            else:
                ref = mp.gammainc(m + mp.mpf(0.5), 0, T) / (2 * mp.power(T, m + mp.mpf(0.5)))
            assert abs(out[m] - float(ref)) <= 2e-14 * float(ref) + 1e-300, (T, m)


def make_shell(am, center, alphas, coefs, keep):
    a = np.array(alphas, dtype=np.float64)
    c = np.array(coefs, dtype=np.float64)
    keep.extend([a, c])
    return Shell(am, len(a), *center, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                 c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))


def quartet(L, s1, s2, s3, s4):
    p1, p2 = Pair(), Pair()
    L.h2g_pair_init(ctypes.byref(p1), ctypes.byref(s1), ctypes.byref(s2))
    L.h2g_pair_init(ctypes.byref(p2), ctypes.byref(s3), ctypes.byref(s4))
    n = [ncart(s.am) for s in (s1, s2, s3, s4)]
    out = np.zeros(int(np.prod(n)))
    L.h2g_eri_quartet(ctypes.byref(p1), ctypes.byref(p2), out.ctypes.data)
    return out.reshape(n)


def test_eri_permutational_symmetry(L):
    keep = []
    rng = np.random.default_rng(0)
    shells = []
    for am in (0, 1, 2, 1):
        c = rng.standard_normal(3)
        a = [2.5, 0.6]
        co = np.array([0.4, 0.7])
        L.h2g_normalize_shell(am, 2, np.array(a).ctypes.data, co.ctypes.data)
        keep.append(co)
        shells.append(make_shell(am, c, a, co, keep))
    A, B, C, D = shells
    abcd = quartet(L, A, B, C, D)
    np.testing.assert_allclose(quartet(L, B, A, C, D), abcd.transpose(1, 0, 2, 3), rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(quartet(L, A, B, D, C), abcd.transpose(0, 1, 3, 2), rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(quartet(L, C, D, A, B), abcd.transpose(2, 3, 0, 1), rtol=1e-11, atol=1e-14)


def test_ssss_closed_form(L):
    keep = []
    a, b = 1.3, 0.4
    sA = make_shell(0, (0.0, 0.0, 0.0), [a], [1.0], keep)
    sB = make_shell(0, (0.0, 0.0, 1.1), [b], [1.0], keep)
    v = quartet(L, sA, sA, sB, sB)[0, 0, 0, 0]
    # (aa|bb) for unnormalised s Gaussians: 2 pi^2.5 / (p q sqrt(p+q)) F0(rho R^2)
    from math import erf, pi, sqrt
    p, q = 2 * a, 2 * b
    rho = p * q / (p + q)
    T = rho * 1.1 ** 2
    F0 = 0.5 * sqrt(pi / T) * erf(sqrt(T))
    ref = 2 * pi ** 2.5 / (p * q * sqrt(p + q)) * F0
    assert abs(v - ref) < 1e-13 * ref


def test_eri_contraction_is_sum_of_primitive_quartets(L):
    """Linearity in the contraction: a contracted quartet (here 3 x 3 = 9
    primitive quartets, computed four at a time with one padded batch) equals
    the sum of its single-primitive quartets (computed one at a time)."""
    keep = []
    rng = np.random.default_rng(7)
    cen = [rng.uniform(-1.5, 1.5, 3) for _ in range(4)]
    aA, cA = [4.1, 1.2, 0.35], [0.3, -0.5, 0.8]
    aC, cC = [2.2, 0.9, 0.27], [0.6, 0.4, -0.2]
    B = make_shell(2, cen[1], [0.8], [1.1], keep)
    D = make_shell(0, cen[3], [0.5], [0.9], keep)
    full = quartet(L, make_shell(1, cen[0], aA, cA, keep), B, make_shell(1, cen[2], aC, cC, keep), D)
    parts = np.zeros_like(full)
    for i in range(3):
        for k in range(3):
            parts += quartet(L, make_shell(1, cen[0], [aA[i]], [cA[i]], keep), B,
                             make_shell(1, cen[2], [aC[k]], [cC[k]], keep), D)
    np.testing.assert_allclose(full, parts, rtol=1e-12, atol=1e-14 * np.abs(full).max())


@pytest.mark.parametrize("side", ["bra", "ket"])
def test_single_p_quartet_is_centre_derivative(L, side):
    """(p s|s s) = d/dA (s' s|s s) with s' the s shell of coefficients
    c_k / (2 a_k) (x - A_x) e^(-a r^2) = (1/2a) d/dA_x e^(-a r^2); likewise on
    the ket. Central differences (step 1e-4) against the one-p path."""
    keep = []
    rng = np.random.default_rng(11)
    cen = [rng.uniform(-1.2, 1.2, 3) for _ in range(4)]
    a, c = [3.1, 0.9, 0.31], [0.5, -0.3, 0.7]
    sp = [ci / (2 * ai) for ai, ci in zip(a, c)]
    others = [make_shell(0, cen[k], [1.7, 0.45], [0.6, 0.8], keep) for k in range(3)]
    h = 1e-4
    for d in range(3):
        if side == "bra":
            p_val = quartet(L, make_shell(1, cen[0], a, c, keep), *others)[d, 0, 0, 0]
        else:
            p_val = quartet(L, others[0], others[1], make_shell(1, cen[0], a, c, keep), others[2])[0, 0, d, 0]
        vals = []
        for sgn in (1, -1):
            A = np.array(cen[0], dtype=float)
            A[d] += sgn * h
            s_shell = make_shell(0, A, a, sp, keep)
            if side == "bra":
                vals.append(quartet(L, s_shell, *others)[0, 0, 0, 0])
            else:
                vals.append(quartet(L, others[0], others[1], s_shell, others[2])[0, 0, 0, 0])
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(p_val - fd) < 1e-7 * max(abs(p_val), 1e-3), (d, p_val, fd)
