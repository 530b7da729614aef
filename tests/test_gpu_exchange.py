"""GPU exchange (K) build through the C ABI, checked against the oracle
(CPU restatement of the reference's H2ERI_build_exchange, pinned to the
reference in test_oracle_pin.py) on the same representation, and against the
reference test suite's golden K.

Tolerance: FP64 path 1e-12 relative (the GPU sums the same products in a
different order: batched over all shell pairs, with atomics)."""
import ctypes
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, relerr

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def oracle_K(oracle_lib, h, D):
    K = np.zeros_like(D)
    oracle_lib.oracle_build_exchange(h.handle, np.ascontiguousarray(D).ctypes.data, K.ctypes.data)
    return K


def test_exchange_golden_and_oracle(alk26, oracle_lib, library):
    """Reference test inputs (tests/test_K_input_mat.c), reference entry point."""
    n = alk26.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk26_ccpvdz.bin")).reshape(n, n)
    Kg = np.fromfile(os.path.join(GOLDEN, "K_alk26_ccpvdz.bin")).reshape(n, n)
    K = np.zeros_like(D)
    library.H2ERI_build_exchange(alk26.handle, D.ctypes.data, K.ctypes.data)
    assert relerr(K, oracle_K(oracle_lib, alk26, D)) < TOL_FP64
    assert relerr(K, Kg) < 5e-6


@pytest.mark.parametrize("name", ["CH4", "C2H6", "C4H10"])
def test_exchange_small_molecules(small_mols, oracle_lib, name):
    """Single leaf (near field only), single level, first admissible pairs."""
    h = small_mols[name]
    D = hg.molecules.seeded_density(h.num_bf, 3, 21)
    assert relerr(h.build_exchange(D), oracle_K(oracle_lib, h, D)) < TOL_FP64


def test_exchange_ranges_and_linearity(alk26, oracle_lib, library):
    """A small work-memory cap splits K into many ranges of n: same K.
    Two densities in one call; K is linear in D."""
    n = alk26.num_bf
    D1 = hg.molecules.seeded_density(n, 33, 2001)
    D2 = hg.molecules.seeded_density(n, 33, 2002)
    K_full = alk26.build_exchange(np.stack([D1, D2, 0.5 * D1 - 2.0 * D2]))
    assert relerr(K_full[0], oracle_K(oracle_lib, alk26, D1)) < TOL_FP64
    assert relerr(K_full[2], 0.5 * K_full[0] - 2.0 * K_full[1]) < 1e-12
    assert library.H2ERI_gpu_set_exchange_memory(alk26.handle, 2e7) == 0
    try:
        K_split = alk26.build_exchange(D1)
        assert alk26.exchange_report()["n_ranges"] > 1
    finally:
        assert library.H2ERI_gpu_set_exchange_memory(alk26.handle, 0) == 0
    assert relerr(K_split, K_full[0]) < TOL_FP64


def test_exchange_device_entry_point(alk32, oracle_lib, library):
    torch = pytest.importorskip("torch")
    n = alk32.num_bf
    D = hg.molecules.seeded_density(n, 20, 78)
    dD = torch.tensor(D, device="cuda")
    dK = torch.empty_like(dD)
    s = torch.cuda.current_stream()
    rc = library.H2ERI_build_exchange_device(alk32.handle, dD.data_ptr(), dK.data_ptr(), ctypes.c_void_p(s.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert relerr(dK.cpu().numpy(), oracle_K(oracle_lib, alk32, D)) < TOL_FP64


def test_exchange_zero_and_screened_density(alk26, oracle_lib):
    """Zero density gives zero K; a density whose off-diagonal shell blocks sit
    below the significance threshold (1e-10) is screened like the reference."""
    n = alk26.num_bf
    assert not np.any(alk26.build_exchange(np.zeros((n, n))))
    D = hg.molecules.seeded_density(n, 12, 5)
    D[np.abs(D) < 0.05] *= 1e-12
    assert relerr(alk26.build_exchange(D), oracle_K(oracle_lib, alk26, D)) < TOL_FP64


def test_exchange_report(alk26):
    alk26.build_exchange(np.eye(alk26.num_bf))
    r = alk26.exchange_report()
    assert r["flops"] > 0 and r["ms_last"] > 0 and r["launches"] >= 3


TOL_MIXED_K = 1e-7   # the H2 tolerance of the exchange configuration (reltol 1e-7)


def test_exchange_mixed_precision(alk26, oracle_lib):
    """FP32 contractions (FP32 blocks, density and work tensors) with FP64
    K assembly, against the FP64 oracle."""
    n = alk26.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk26_ccpvdz.bin")).reshape(n, n)
    K64 = oracle_K(oracle_lib, alk26, D)
    alk26.set_precision(hg.MIXED)
    try:
        K32 = alk26.build_exchange(D)
    finally:
        alk26.set_precision(hg.FP64)
    err = relerr(K32, K64)
    print(f"mixed K relerr vs FP64 oracle: {err:.3e}")
    assert err < TOL_MIXED_K


def test_exchange_mixed_tensor_cores_and_simt(oracle_lib, library, monkeypatch):
    """The mixed mode's products on the tensor cores (FP32 operands split
    into three bf16 parts, six products accumulated in FP32 in tensor memory;
    the persistent warp-specialised kernel and the one-tile-per-CTA kernel,
    H2G_K_TC=2) and on the FP32 SIMT kernel (H2G_K_TC=0) all stay within the exchange
    tolerance of the FP64 oracle, also with the n range split into several
    ranges, and agree with each other to FP32-accumulation level."""
    mol = os.path.join(GOLDEN, "alk26_ccpvdz.mol")
    Ks, hs = {}, {}
    try:
        for flag in ("1", "2", "0"):
            monkeypatch.setenv("H2G_K_TC", flag)
            h = hs[flag] = hg.H2ERI.from_mol(mol, qr_tol=1e-6)
            n = h.num_bf
            D = hg.molecules.seeded_density(n, 33, 2101)
            h.set_precision(hg.MIXED)
            Ks[flag] = h.build_exchange(D)
            assert h.exchange_report()["tensor_cores"] == float(flag != "0")
            assert library.H2ERI_gpu_set_exchange_memory(h.handle, 2e7) == 0
            K_split = h.build_exchange(D)
            assert h.exchange_report()["n_ranges"] > 1
            assert relerr(K_split, Ks[flag]) < 1e-8
        K64 = oracle_K(oracle_lib, hs["1"], D)
        e_tc, e_tile, e_simt = relerr(Ks["1"], K64), relerr(Ks["2"], K64), relerr(Ks["0"], K64)
        print(f"mixed K relerr vs FP64 oracle: tensor cores {e_tc:.3e} (one tile per CTA {e_tile:.3e}), "
              f"FP32 SIMT {e_simt:.3e}")
        assert e_tc < TOL_MIXED_K and e_tile < TOL_MIXED_K and e_simt < TOL_MIXED_K
        assert relerr(Ks["1"], Ks["0"]) < TOL_MIXED_K
        # the two tensor-core kernels form the same tile products (their FP32
        # atomics into the work tensors land in a different order)
        assert relerr(Ks["1"], Ks["2"]) < TOL_MIXED_K
    finally:
        for h in hs.values():
            h.destroy()


@pytest.mark.slow
def test_exchange_3d_methane_cluster(library, oracle_lib, tmp_path):
    """A 3-D system: 8 CH4 on a jittered 2 x 2 x 2 lattice (4.0 A, random
    orientations; 280 Cartesian bf), QR tolerance 1e-7. Every molecule has
    neighbours on all sides, so nodes carry far more coupling and near-field
    work than on a chain. FP64 K against the oracle at 1e-12, mixed K at
    1e-7."""
    p = str(tmp_path / "ch4x8.mol")
    hg.molecules.write_methane_cluster(p, shape=(2, 2, 2))
    h = hg.H2ERI.from_mol(p, qr_tol=1e-7)
    try:
        n = h.num_bf
        D = hg.molecules.seeded_density(n, 40, 5000)
        Ko = oracle_K(oracle_lib, h, D)
        K64 = h.build_exchange(D)
        h.set_precision(hg.MIXED)
        try:
            Km = h.build_exchange(D)
        finally:
            h.set_precision(hg.FP64)
        e64, em = relerr(K64, Ko), relerr(Km, Ko)
        print(f"(CH4)8 3-D cluster K: FP64 {e64:.2e}, mixed {em:.2e}")
        assert e64 < TOL_FP64
        assert em < TOL_MIXED_K
    finally:
        h.destroy()
