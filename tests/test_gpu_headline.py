"""The benchmark configurations under the GPU parity suite, not only inside
the benchmark: straight-chain alkanes C30H62 (760 Cartesian basis functions)
and C100H202 (2510) at QR tolerance 1e-8, seeded densities, every result
checked against the FP64 oracle on the same representation.

  FP64 J                      <= 1e-12 relative (reference entry point)
  mixed J, one density        <= 1e-8
  mixed J, 16 densities in
  one launch                  <= 1e-8 for every one of the 16
  K at QR tolerance 1e-7      FP64 <= 1e-12, mixed <= 1e-7 (C10H22; the oracle's
                              K of C30H62 takes minutes on the host cores)

The set-up of C100H202 takes about a minute of host time."""
import ctypes
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import relerr

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
N_DEN = 16


def _alkane(tmp_path_factory, n, qr):
    p = str(tmp_path_factory.mktemp(f"c{n}") / f"alk{n}.mol")
    hg.molecules.write_alkane(p, n)
    return hg.H2ERI.from_mol(p, qr_tol=qr)


@pytest.fixture(scope="module")
def c30(library, tmp_path_factory):
    h = _alkane(tmp_path_factory, 30, 1e-8)
    yield h
    h.destroy()


@pytest.fixture(scope="module")
def c100(library, tmp_path_factory):
    h = _alkane(tmp_path_factory, 100, 1e-8)
    yield h
    h.destroy()


def oracle_J(oracle_lib, h, D):
    J = np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(h.handle, np.ascontiguousarray(D).ctypes.data, J.ctypes.data)
    return J


def _check_alkane(h, oracle_lib, library, n_occ, seed):
    torch = pytest.importorskip("torch")
    n = h.num_bf
    D = hg.molecules.seeded_density(n, n_occ, seed)
    Jo = oracle_J(oracle_lib, h, D)
    h.set_precision(hg.FP64)
    J = np.zeros_like(D)
    library.H2ERI_build_Coulomb(h.handle, D.ctypes.data, J.ctypes.data)
    e64 = relerr(J, Jo)
    h.set_precision(hg.MIXED)
    try:
        Jm = np.zeros_like(D)
        library.H2ERI_build_Coulomb(h.handle, D.ctypes.data, Jm.ctypes.data)
        em = relerr(Jm, Jo)
        Ds = np.stack([hg.molecules.seeded_density(n, n_occ, seed + 100 + i) for i in range(N_DEN)])
        dD = torch.tensor(Ds, device="cuda")
        dJ = torch.full_like(dD, float("nan"))
        s = torch.cuda.current_stream()
        rc = library.H2ERI_build_Coulomb_device(h.handle, N_DEN, dD.data_ptr(), dJ.data_ptr(),
                                                ctypes.c_void_p(s.cuda_stream))
        assert rc == 0, library.H2ERI_gpu_last_error()
        torch.cuda.synchronize()
        J16 = dJ.cpu().numpy()
    finally:
        h.set_precision(hg.FP64)
    e16 = [relerr(J16[i], oracle_J(oracle_lib, h, Ds[i])) for i in range(N_DEN)]
    print(f"{n} bf: FP64 J {e64:.2e}, mixed J {em:.2e}, {N_DEN} densities per launch max {max(e16):.2e}")
    assert e64 < 1e-12
    assert em < 1e-8
    assert max(e16) < 1e-8, e16


def test_c30h62_fp64_mixed_and_16_densities(c30, oracle_lib, library):
    _check_alkane(c30, oracle_lib, library, 121, 2000)


def test_c100h202_fp64_mixed_and_16_densities(c100, oracle_lib, library):
    _check_alkane(c100, oracle_lib, library, 401, 3000)


def test_exchange_at_qr_1e7(library, oracle_lib, tmp_path_factory):
    h = _alkane(tmp_path_factory, 10, 1e-7)
    try:
        n = h.num_bf
        D = hg.molecules.seeded_density(n, 41, 5000)
        Ko = np.zeros_like(D)
        oracle_lib.oracle_build_exchange(h.handle, D.ctypes.data, Ko.ctypes.data)
        K64 = h.build_exchange(D)
        h.set_precision(hg.MIXED)
        try:
            Km = h.build_exchange(D)
        finally:
            h.set_precision(hg.FP64)
        e64, em = relerr(K64, Ko), relerr(Km, Ko)
        print(f"C10H22 QR 1e-7 K: FP64 {e64:.2e}, mixed {em:.2e}")
        assert e64 < 1e-12
        assert em < 1e-7
    finally:
        h.destroy()
