"""Pins the oracle (CPU restatement of the hot path) to the reference: the
reference's own compiled H2ERI_matvec / H2ERI_build_Coulomb on the same struct
(where the reference sources exist), and the reference test suite's golden J."""
import ctypes
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, ref_lib_or_skip, relerr


def test_oracle_J_matches_golden(alk32, oracle_lib):
    n = alk32.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk32_ccpvdz.bin")).reshape(n, n)
    Jg = np.fromfile(os.path.join(GOLDEN, "J_alk32_ccpvdz.bin")).reshape(n, n)
    J = np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(alk32.handle, D.ctypes.data, J.ctypes.data)
    assert relerr(J, Jg) < 2e-7
    np.testing.assert_allclose(J, J.T, rtol=0, atol=1e-13 * np.abs(J).max())


def test_oracle_matvec_equals_reference_on_native_rep(alk32, oracle_lib):
    ref = ref_lib_or_skip()
    rng = np.random.default_rng(7)
    x = rng.standard_normal(alk32.krnl_mat_size)
    y_o = np.zeros_like(x)
    y_r = np.zeros_like(x)
    oracle_lib.oracle_matvec(alk32.handle, x.ctypes.data, y_o.ctypes.data)
    ref.H2ERI_matvec(alk32.handle, x.ctypes.data, y_r.ctypes.data)
    assert relerr(y_o, y_r) < 1e-13


def test_oracle_matvec_equals_reference_on_reference_rep(oracle_lib):
    """Both run on the representation built by the reference's own set-up."""
    ref = ref_lib_or_skip()
    rh = ref.oref_build(os.path.join(GOLDEN, "alk26_ccpvdz.mol").encode(), 1e-10, 1e-10, 1e-6, 0)
    krnl = ctypes.cast(rh, ctypes.POINTER(hg.H2ERIStruct)).contents.krnl_mat_size
    rng = np.random.default_rng(11)
    for _ in range(2):
        x = rng.standard_normal(krnl)
        y_o = np.zeros_like(x)
        y_r = np.zeros_like(x)
        oracle_lib.oracle_matvec(rh, x.ctypes.data, y_o.ctypes.data)
        ref.H2ERI_matvec(rh, x.ctypes.data, y_r.ctypes.data)
        assert relerr(y_o, y_r) < 1e-13


def test_oracle_coulomb_equals_reference(alk32, oracle_lib):
    ref = ref_lib_or_skip()
    n = alk32.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk32_ccpvdz.bin")).reshape(n, n)
    J_o = np.zeros_like(D)
    J_r = np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(alk32.handle, D.ctypes.data, J_o.ctypes.data)
    ref.H2ERI_build_Coulomb(alk32.handle, D.ctypes.data, J_r.ctypes.data)
    assert relerr(J_o, J_r) < 1e-13


def test_oracle_linearity(alk26, oracle_lib):
    rng = np.random.default_rng(3)
    k = alk26.krnl_mat_size
    a, b = rng.standard_normal(k), rng.standard_normal(k)
    ya, yb, yab = (np.zeros(k) for _ in range(3))
    c = 0.37
    ab = a + c * b
    oracle_lib.oracle_matvec(alk26.handle, a.ctypes.data, ya.ctypes.data)
    oracle_lib.oracle_matvec(alk26.handle, b.ctypes.data, yb.ctypes.data)
    oracle_lib.oracle_matvec(alk26.handle, ab.ctypes.data, yab.ctypes.data)
    assert relerr(yab, ya + c * yb) < 1e-13


def test_oracle_K_equals_reference_on_reference_rep(oracle_lib):
    """Exchange: oracle restatement vs the reference's own H2ERI_build_exchange
    on the representation built by the reference's set-up."""
    ref = ref_lib_or_skip()
    rh = ref.oref_build(os.path.join(GOLDEN, "alk26_ccpvdz.mol").encode(), 1e-10, 1e-10, 1e-6, 0)
    n = 210
    D = np.fromfile(os.path.join(GOLDEN, "D_alk26_ccpvdz.bin")).reshape(n, n)
    K_o = np.zeros_like(D)
    K_r = np.zeros_like(D)
    oracle_lib.oracle_build_exchange(rh, D.ctypes.data, K_o.ctypes.data)
    ref.H2ERI_build_exchange(rh, D.ctypes.data, K_r.ctypes.data)
    assert relerr(K_o, K_r) < 1e-13


def test_oracle_K_matches_golden(alk26, oracle_lib):
    """K of the reference test suite (tests/test_K_input_mat.c inputs), on the
    native representation at QR tol 1e-6."""
    n = alk26.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk26_ccpvdz.bin")).reshape(n, n)
    Kg = np.fromfile(os.path.join(GOLDEN, "K_alk26_ccpvdz.bin")).reshape(n, n)
    K = np.zeros_like(D)
    oracle_lib.oracle_build_exchange(alk26.handle, D.ctypes.data, K.ctypes.data)
    assert relerr(K, Kg) < 5e-6


def test_reference_fixture_loads_and_oracle_reproduces_it(oracle_lib):
    """The committed fixture made by the reference itself (its own set-up,
    matvec, J and K on a 40-atom hydrogen chain, tests/golden/
    make_ref_fixture.py): the representation loads, and the oracle on it
    reproduces the reference's numbers. The GPU tests compare with the same
    numbers directly."""
    h = hg.H2ERI.load(os.path.join(GOLDEN, "ref_h40.h2r"))
    try:
        n = h.num_bf
        x = np.fromfile(os.path.join(GOLDEN, "ref_h40_x.bin"))
        assert x.size == h.krnl_mat_size
        y = np.zeros_like(x)
        oracle_lib.oracle_matvec(h.handle, x.ctypes.data, y.ctypes.data)
        assert relerr(y, np.fromfile(os.path.join(GOLDEN, "ref_h40_y.bin"))) < 1e-13
        D = np.fromfile(os.path.join(GOLDEN, "ref_h40_D.bin")).reshape(n, n)
        J = np.zeros_like(D)
        K = np.zeros_like(D)
        oracle_lib.oracle_build_Coulomb(h.handle, D.ctypes.data, J.ctypes.data)
        oracle_lib.oracle_build_exchange(h.handle, D.ctypes.data, K.ctypes.data)
        assert relerr(J, np.fromfile(os.path.join(GOLDEN, "ref_h40_J.bin")).reshape(n, n)) < 1e-13
        assert relerr(K, np.fromfile(os.path.join(GOLDEN, "ref_h40_K.bin")).reshape(n, n)) < 1e-13
    finally:
        h.destroy()
