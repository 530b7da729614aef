"""Mixed-precision far field / near field on the GPU: U bases as FP32 pairs,
B and D blocks as FP32, compensated FP32 products, FP64 reductions. Checked
against the FP64 oracle on the same representation; tolerance 1e-8 relative
(the target accuracy of the mixed mode)."""
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, relerr

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-8


def oracle_J(oracle_lib, h, D):
    J = np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(h.handle, np.ascontiguousarray(D).ctypes.data, J.ctypes.data)
    return J


def test_mixed_coulomb_alk32(alk32, oracle_lib):
    n = alk32.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk32_ccpvdz.bin")).reshape(n, n)
    Jo = oracle_J(oracle_lib, alk32, D)
    alk32.set_precision(hg.MIXED)
    try:
        J = alk32.build_coulomb(D)
        assert alk32.report()["precision"] == hg.MIXED
    finally:
        alk32.set_precision(hg.FP64)
    e = relerr(J, Jo)
    assert e < TOL_MIXED, e
    assert e > 1e-14      # the FP32 blocks really are in use
    np.testing.assert_array_equal(J, J.T)
    # back in FP64 mode the FP64 tolerance holds again
    assert relerr(alk32.build_coulomb(D), Jo) < 1e-12


# For random (structureless) vectors A x cancels far more than for a density,
# so the FP32 storage rounding (2^-24 relative per entry) shows up as ~1e-7
# relative error; the 1e-8 target applies to J builds from densities.
TOL_MIXED_RANDOM = 5e-7


def test_mixed_matvec_multi(alk26, oracle_lib):
    rng = np.random.default_rng(21)
    X = rng.standard_normal((2, alk26.krnl_mat_size))
    alk26.set_precision(hg.MIXED)
    try:
        Y = alk26.matvec(X)
    finally:
        alk26.set_precision(hg.FP64)
    for i in range(2):
        yo = np.zeros_like(X[i])
        oracle_lib.oracle_matvec(alk26.handle, X[i].ctypes.data, yo.ctypes.data)
        assert relerr(Y[i], yo) < TOL_MIXED_RANDOM


@pytest.mark.parametrize("name", ["CH4", "C2H6", "C4H10"])
def test_mixed_small_molecules(small_mols, oracle_lib, name):
    h = small_mols[name]
    D = hg.molecules.seeded_density(h.num_bf, 3, 19)
    h.set_precision(hg.MIXED)
    try:
        J = h.build_coulomb(D)
    finally:
        h.set_precision(hg.FP64)
    assert relerr(J, oracle_J(oracle_lib, h, D)) < TOL_MIXED
