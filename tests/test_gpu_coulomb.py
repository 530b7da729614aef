"""GPU hot path through the C ABI, checked against the oracle (CPU
restatement of the reference, pinned in test_oracle_pin.py) on the same
representation, and against the reference test suite's golden J.

Tolerances: FP64 path 1e-12 relative (GPU atomics sum in a different order
than the CPU threads; nothing else differs)."""
import ctypes
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, relerr

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def oracle_matvec(oracle_lib, h, x):
    y = np.zeros_like(x)
    oracle_lib.oracle_matvec(h.handle, x.ctypes.data, y.ctypes.data)
    return y


def oracle_J(oracle_lib, h, D):
    J = np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(h.handle, np.ascontiguousarray(D).ctypes.data, J.ctypes.data)
    return J


def test_matvec_matches_oracle_alk32(alk32, oracle_lib):
    rng = np.random.default_rng(1)
    for _ in range(3):
        x = rng.standard_normal(alk32.krnl_mat_size)
        y = alk32.matvec(x)
        assert relerr(y, oracle_matvec(oracle_lib, alk32, x)) < TOL_FP64


def test_reference_entry_point_matvec(alk32, oracle_lib, library):
    """H2ERI_matvec with the reference signature (host pointers)."""
    x = np.random.default_rng(2).standard_normal(alk32.krnl_mat_size)
    y = np.zeros_like(x)
    library.H2ERI_matvec(alk32.handle, x.ctypes.data, y.ctypes.data)
    assert relerr(y, oracle_matvec(oracle_lib, alk32, x)) < TOL_FP64


def test_coulomb_golden_and_oracle(alk32, oracle_lib, library):
    n = alk32.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk32_ccpvdz.bin")).reshape(n, n)
    Jg = np.fromfile(os.path.join(GOLDEN, "J_alk32_ccpvdz.bin")).reshape(n, n)
    J = np.zeros_like(D)
    library.H2ERI_build_Coulomb(alk32.handle, D.ctypes.data, J.ctypes.data)
    assert relerr(J, oracle_J(oracle_lib, alk32, D)) < TOL_FP64
    assert relerr(J, Jg) < 2e-7
    np.testing.assert_array_equal(J, J.T)


def test_matvec_multi_vector(alk26, oracle_lib):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((3, alk26.krnl_mat_size))
    Y = alk26.matvec(X)
    for i in range(3):
        assert relerr(Y[i], oracle_matvec(oracle_lib, alk26, X[i].copy())) < TOL_FP64


def test_coulomb_multi_density_and_linearity(alk26, oracle_lib):
    n = alk26.num_bf
    D1 = hg.molecules.seeded_density(n, 33, 1001)
    D2 = hg.molecules.seeded_density(n, 33, 1002)
    J = alk26.build_coulomb(np.stack([D1, D2, 0.5 * D1 - 2.0 * D2]))
    assert relerr(J[0], oracle_J(oracle_lib, alk26, D1)) < TOL_FP64
    assert relerr(J[1], oracle_J(oracle_lib, alk26, D2)) < TOL_FP64
    assert relerr(J[2], 0.5 * J[0] - 2.0 * J[1]) < 1e-12


def test_device_entry_point(alk26, oracle_lib, library):
    torch = pytest.importorskip("torch")
    n = alk26.num_bf
    D = hg.molecules.seeded_density(n, 20, 77)
    dD = torch.tensor(D, device="cuda")
    dJ = torch.empty_like(dD)
    s = torch.cuda.current_stream()
    rc = library.H2ERI_build_Coulomb_device(alk26.handle, 1, dD.data_ptr(), dJ.data_ptr(), ctypes.c_void_p(s.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert relerr(dJ.cpu().numpy(), oracle_J(oracle_lib, alk26, D)) < TOL_FP64


def test_coulomb_page_locked_host_buffers(alk26, oracle_lib, library):
    """Page-locked caller buffers are read and written in place by the
    kernels; pageable ones go through staging copies. Every combination gives
    the oracle's J, for one and for several densities."""
    torch = pytest.importorskip("torch")
    n = alk26.num_bf
    Ds = np.stack([hg.molecules.seeded_density(n, 20, 90 + i) for i in range(3)])
    Jo = [oracle_J(oracle_lib, alk26, Ds[i]) for i in range(3)]
    pinD = torch.from_numpy(Ds.copy()).pin_memory()
    for d_pinned in (True, False):
        for j_pinned in (True, False):
            srcD = pinD if d_pinned else torch.from_numpy(Ds.copy())
            dstJ = torch.zeros(3, n, n, dtype=torch.float64, pin_memory=j_pinned)
            rc = library.H2ERI_build_Coulomb_multi(alk26.handle, 3, srcD.data_ptr(), dstJ.data_ptr())
            assert rc == 0, (d_pinned, j_pinned)
            for i in range(3):
                assert relerr(dstJ[i].numpy(), Jo[i]) < TOL_FP64, (d_pinned, j_pinned, i)
    # a single density out of a larger page-locked buffer (offset view)
    J1 = torch.zeros(n, n, dtype=torch.float64, pin_memory=True)
    rc = library.H2ERI_build_Coulomb_multi(alk26.handle, 1, pinD[1].data_ptr(), J1.data_ptr())
    assert rc == 0
    assert relerr(J1.numpy(), Jo[1]) < TOL_FP64


@pytest.mark.parametrize("name", ["CH4", "C2H6", "C4H10"])
def test_small_molecules(small_mols, oracle_lib, name):
    """Single-leaf (no far field), single-level and first-admissible trees."""
    h = small_mols[name]
    x = np.random.default_rng(5).standard_normal(h.krnl_mat_size)
    assert relerr(h.matvec(x), oracle_matvec(oracle_lib, h, x)) < TOL_FP64
    D = hg.molecules.seeded_density(h.num_bf, 3, 9)
    assert relerr(h.build_coulomb(D), oracle_J(oracle_lib, h, D)) < TOL_FP64


def test_loaded_representation(alk26, oracle_lib, tmp_path):
    p = str(tmp_path / "rep.h2r")
    alk26.save(p)
    h2 = hg.H2ERI.load(p)
    try:
        x = np.random.default_rng(6).standard_normal(alk26.krnl_mat_size)
        assert relerr(h2.matvec(x), oracle_matvec(oracle_lib, alk26, x)) < TOL_FP64
    finally:
        h2.destroy()


def test_zero_density_and_repeat(alk26):
    n = alk26.num_bf
    J0 = alk26.build_coulomb(np.zeros((n, n)))
    assert not np.any(J0)
    D = hg.molecules.seeded_density(n, 10, 12)
    Ja = alk26.build_coulomb(D)
    Jb = alk26.build_coulomb(D)
    assert relerr(Ja, Jb) < 1e-14


def test_bad_arguments_return_errors(alk26, library):
    x = np.zeros(alk26.krnl_mat_size)
    assert library.H2ERI_matvec_multi(alk26.handle, 0, x.ctypes.data, x.ctypes.data) != 0
    assert b"nvec" in library.H2ERI_gpu_last_error()
    assert library.H2ERI_gpu_set_precision(alk26.handle, 7) != 0


def test_timers_and_report(alk26):
    alk26.build_coulomb(np.eye(alk26.num_bf))
    r = alk26.report()
    assert r["launches_per_matvec"] >= 3
    assert r["alg_matrix_bytes"] > 0 and r["ms_total"] > 0
    assert alk26.s.timers[7] > 0.0   # near-field phase time filled from CUDA events


def test_coulomb_batch_of_molecules(small_mols, alk32, oracle_lib, library):
    """Several structures of different sizes in one batched call (their
    builds run concurrently on their own streams): every J matches the oracle."""
    torch = pytest.importorskip("torch")
    hs = [small_mols["C2H6"], small_mols["C4H10"], alk32]
    nd = [2, 3, 2]
    dens, dDs, dJs = [], [], []
    for k, (h, n) in enumerate(zip(hs, nd)):
        D = np.stack([hg.molecules.seeded_density(h.num_bf, 3 + k, 400 + 10 * k + i) for i in range(n)])
        dens.append(D)
        dDs.append(torch.tensor(D, device="cuda"))
        dJs.append(torch.zeros_like(dDs[-1]))
    harr = (ctypes.c_void_p * 3)(*[h.handle.value for h in hs])
    narr = (ctypes.c_int * 3)(*nd)
    darr = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in dDs])
    jarr = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in dJs])
    s = torch.cuda.current_stream()
    rc = library.H2ERI_build_Coulomb_batch(3, harr, narr, darr, jarr, ctypes.c_void_p(s.cuda_stream))
    assert rc == 0, library.H2ERI_gpu_last_error()
    torch.cuda.synchronize()
    for h, D, dJ in zip(hs, dens, dJs):
        J = dJ.cpu().numpy()
        for i in range(D.shape[0]):
            Jo = np.zeros_like(D[i])
            oracle_lib.oracle_build_Coulomb(h.handle, np.ascontiguousarray(D[i]).ctypes.data, Jo.ctypes.data)
            assert relerr(J[i], Jo) < 1e-12
    # a structure may appear only once per call
    harr2 = (ctypes.c_void_p * 2)(hs[0].handle.value, hs[0].handle.value)
    assert library.H2ERI_build_Coulomb_batch(2, harr2, narr, darr, jarr, ctypes.c_void_p(s.cuda_stream)) != 0
