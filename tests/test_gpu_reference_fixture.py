"""GPU results against numbers the reference itself produced (no oracle in
between): the representation of a 40-atom hydrogen chain built by the
reference's own set-up, and its H2ERI_matvec, H2ERI_build_Coulomb and
H2ERI_build_exchange outputs on a seeded vector and density
(tests/golden/make_ref_fixture.py). The GPU path loads the same
representation and is called through the reference's entry points.

Tolerances: FP64 1e-12 relative; mixed mode J 1e-8 (its target accuracy),
mixed K 1e-7 (the H2 tolerance of the exchange configuration)."""
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, relerr

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


@pytest.fixture(scope="module")
def ref_h40(library):
    h = hg.H2ERI.load(os.path.join(GOLDEN, "ref_h40.h2r"))
    yield h
    h.destroy()


def _golden(name, shape=None):
    a = np.fromfile(os.path.join(GOLDEN, f"ref_h40_{name}.bin"))
    return a.reshape(shape) if shape else a


def test_fp64_matches_reference_outputs(ref_h40, library):
    n = ref_h40.num_bf
    ref_h40.set_precision(hg.FP64)
    x = _golden("x")
    y = np.zeros_like(x)
    library.H2ERI_matvec(ref_h40.handle, x.ctypes.data, y.ctypes.data)
    assert relerr(y, _golden("y")) < TOL_FP64
    D = _golden("D", (n, n))
    J = np.zeros_like(D)
    K = np.zeros_like(D)
    library.H2ERI_build_Coulomb(ref_h40.handle, D.ctypes.data, J.ctypes.data)
    library.H2ERI_build_exchange(ref_h40.handle, D.ctypes.data, K.ctypes.data)
    eJ, eK = relerr(J, _golden("J", (n, n))), relerr(K, _golden("K", (n, n)))
    print(f"reference-built H40, FP64: matvec {relerr(y, _golden('y')):.2e}, J {eJ:.2e}, K {eK:.2e}")
    assert eJ < TOL_FP64 and eK < TOL_FP64


def test_mixed_matches_reference_outputs(ref_h40, library):
    n = ref_h40.num_bf
    D = _golden("D", (n, n))
    ref_h40.set_precision(hg.MIXED)
    try:
        J = np.zeros_like(D)
        K = np.zeros_like(D)
        library.H2ERI_build_Coulomb(ref_h40.handle, D.ctypes.data, J.ctypes.data)
        library.H2ERI_build_exchange(ref_h40.handle, D.ctypes.data, K.ctypes.data)
    finally:
        ref_h40.set_precision(hg.FP64)
    eJ, eK = relerr(J, _golden("J", (n, n))), relerr(K, _golden("K", (n, n)))
    print(f"reference-built H40, mixed: J {eJ:.2e}, K {eK:.2e}")
    assert eJ < 1e-8
    assert eK < 1e-7
