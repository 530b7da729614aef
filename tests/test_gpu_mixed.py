"""Mixed precision on the GPU: U bases and leaf self-interaction D blocks as
FP32 pairs, other B and D blocks as FP32, products accumulated in anchored
FP32 chains, FP64 output sums. Checked against the FP64 oracle on the same
representation through every entry point; tolerance 1e-8 relative (the
target accuracy of the mixed mode)."""
import ctypes
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


def test_mixed_device_multi_density_and_linearity(alk26, oracle_lib, library):
    """Several densities per launch on device arrays: each J within 1e-8 of
    the oracle, and the build stays linear in the density to that level."""
    torch = pytest.importorskip("torch")
    n = alk26.num_bf
    D1 = hg.molecules.seeded_density(n, 33, 3101)
    D2 = hg.molecules.seeded_density(n, 33, 3102)
    Ds = np.stack([D1, D2, 0.5 * D1 - 2.0 * D2])
    dD = torch.tensor(Ds, device="cuda")
    dJ = torch.zeros_like(dD)
    alk26.set_precision(hg.MIXED)
    try:
        s = torch.cuda.current_stream()
        rc = library.H2ERI_build_Coulomb_device(alk26.handle, 3, dD.data_ptr(), dJ.data_ptr(),
                                                ctypes.c_void_p(s.cuda_stream))
        assert rc == 0, library.H2ERI_gpu_last_error()
        torch.cuda.synchronize()
    finally:
        alk26.set_precision(hg.FP64)
    J = dJ.cpu().numpy()
    for i in range(3):
        assert relerr(J[i], oracle_J(oracle_lib, alk26, Ds[i])) < TOL_MIXED, i
    assert relerr(J[2], 0.5 * J[0] - 2.0 * J[1]) < TOL_MIXED


def test_mixed_noalloc_matches_device_entry_point(alk26, library):
    """The allocation-free matvec runs the same mixed kernels."""
    torch = pytest.importorskip("torch")
    alk26.set_precision(hg.MIXED)
    try:
        s = torch.cuda.Stream()
        sp = ctypes.c_void_p(s.cuda_stream)
        x = torch.tensor(np.random.default_rng(77).standard_normal(alk26.krnl_mat_size), device="cuda")
        y_ref = torch.empty_like(x)
        y = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        assert library.H2ERI_matvec_device(alk26.handle, 1, x.data_ptr(), y_ref.data_ptr(), sp) == 0
        rc = library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), sp)
        assert rc == 0, library.H2ERI_gpu_last_error()
        s.synchronize()
    finally:
        alk26.set_precision(hg.FP64)
    # same kernels; only the order of the FP64 atomic additions differs
    assert relerr(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-12


def test_mixed_batch_and_page_locked_buffers(small_mols, alk32, oracle_lib, library):
    """The batched call and the page-locked host path in mixed mode."""
    torch = pytest.importorskip("torch")
    hs = [small_mols["C4H10"], alk32]
    dens = [np.stack([hg.molecules.seeded_density(h.num_bf, 4 + k, 700 + 10 * k + i) for i in range(2)])
            for k, h in enumerate(hs)]
    for h in hs:
        h.set_precision(hg.MIXED)
    try:
        dDs = [torch.tensor(D, device="cuda") for D in dens]
        dJs = [torch.zeros_like(t) for t in dDs]
        harr = (ctypes.c_void_p * 2)(*[h.handle.value for h in hs])
        narr = (ctypes.c_int * 2)(2, 2)
        darr = (ctypes.c_void_p * 2)(*[t.data_ptr() for t in dDs])
        jarr = (ctypes.c_void_p * 2)(*[t.data_ptr() for t in dJs])
        s = torch.cuda.current_stream()
        rc = library.H2ERI_build_Coulomb_batch(2, harr, narr, darr, jarr, ctypes.c_void_p(s.cuda_stream))
        assert rc == 0, library.H2ERI_gpu_last_error()
        torch.cuda.synchronize()
        pD = torch.from_numpy(dens[1].copy()).pin_memory()
        pJ = torch.zeros(pD.shape, dtype=torch.float64, pin_memory=True)
        assert library.H2ERI_build_Coulomb_multi(alk32.handle, 2, pD.data_ptr(), pJ.data_ptr()) == 0
    finally:
        for h in hs:
            h.set_precision(hg.FP64)
    for h, D, dJ in zip(hs, dens, dJs):
        J = dJ.cpu().numpy()
        for i in range(2):
            assert relerr(J[i], oracle_J(oracle_lib, h, D[i])) < TOL_MIXED
    for i in range(2):
        assert relerr(pJ[i].numpy(), oracle_J(oracle_lib, alk32, dens[1][i])) < TOL_MIXED


def test_precision_from_environment(tmp_path, oracle_lib, library, monkeypatch):
    """H2G_PRECISION=mixed starts a structure in the mixed mode, so callers of
    the reference entry points alone get it; an unknown value is an error."""
    p = str(tmp_path / "c4h10.mol")
    hg.molecules.write_alkane(p, 4)
    monkeypatch.setenv("H2G_PRECISION", "mixed")
    h = hg.H2ERI.from_mol(p, qr_tol=1e-8)
    try:
        D = hg.molecules.seeded_density(h.num_bf, 4, 808)
        J = np.zeros_like(D)
        library.H2ERI_build_Coulomb(h.handle, D.ctypes.data, J.ctypes.data)   # reference signature
        assert h.report()["precision"] == hg.MIXED
        e = relerr(J, oracle_J(oracle_lib, h, D))
        assert 1e-14 < e < TOL_MIXED, e
    finally:
        h.destroy()
    monkeypatch.setenv("H2G_PRECISION", "fp32")
    h = hg.H2ERI.from_mol(p, qr_tol=1e-8)
    try:
        D = hg.molecules.seeded_density(h.num_bf, 4, 808)
        J = np.zeros_like(D)
        assert library.H2ERI_build_Coulomb_multi(h.handle, 1, D.ctypes.data, J.ctypes.data) != 0
        assert b"H2G_PRECISION" in library.H2ERI_gpu_last_error()
    finally:
        h.destroy()


def test_batch_in_shared_launches(small_mols, alk26, alk32, oracle_lib, library, monkeypatch):
    """Five structures of different sizes, two densities each, in one
    H2ERI_build_Coulomb_batch call in the mixed mode: their tiles run in
    shared tensor-core launches, phase by phase (one launch carries tiles of
    every structure). Every J matches the FP64 oracle to the mixed-mode
    tolerance and the per-structure path (each structure on its own streams,
    H2G_BATCH_MERGED=0) to 1e-12: the same kernel, only the order of the
    output atomics differs. A second call reuses the batch plan."""
    torch = pytest.importorskip("torch")
    hs = [small_mols["CH4"], small_mols["C2H6"], small_mols["C4H10"], alk26, alk32]
    n = len(hs)
    dens = [np.stack([hg.molecules.seeded_density(h.num_bf, 3 + k, 900 + 10 * k + i) for i in range(2)])
            for k, h in enumerate(hs)]
    for h in hs:
        h.set_precision(hg.MIXED)
    try:
        dDs = [torch.tensor(D, device="cuda") for D in dens]
        harr = (ctypes.c_void_p * n)(*[h.handle.value for h in hs])
        narr = (ctypes.c_int * n)(*([2] * n))
        darr = (ctypes.c_void_p * n)(*[t.data_ptr() for t in dDs])
        s = torch.cuda.current_stream()
        out = {}
        for mode in ("1", "0", "1"):
            monkeypatch.setenv("H2G_BATCH_MERGED", mode)
            dJs = [torch.full_like(t, float("nan")) for t in dDs]
            jarr = (ctypes.c_void_p * n)(*[t.data_ptr() for t in dJs])
            rc = library.H2ERI_build_Coulomb_batch(n, harr, narr, darr, jarr, ctypes.c_void_p(s.cuda_stream))
            assert rc == 0, library.H2ERI_gpu_last_error()
            torch.cuda.synchronize()
            out.setdefault(mode, []).append([t.cpu().numpy() for t in dJs])
        assert all(library.H2ERI_gpu_check(h.handle) == 0 for h in hs)
    finally:
        for h in hs:
            h.set_precision(hg.FP64)
    merged, single = out["1"][0], out["0"][0]
    for k, h in enumerate(hs):
        for i in range(2):
            assert relerr(merged[k][i], oracle_J(oracle_lib, h, dens[k][i])) < TOL_MIXED, (k, i)
            assert relerr(merged[k][i], single[k][i]) < 1e-12, (k, i)
            assert relerr(out["1"][1][k][i], merged[k][i]) < 1e-12, (k, i)


def test_batch_in_shared_launches_single_density_kernels(oracle_lib, library, monkeypatch, tmp_path):
    """The same shared-launch batch when the structures' launch choices put
    two densities on the single-density kernels (as the tuner does for
    short chains): their tile plans are merged phase by phase for the mixed
    tile kernel, with the tensor maps of all structures in one array. Tile
    shapes differ between structures (256 and 512 rows)."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("H2G_MMA_MIN_VEC", "3")
    hs = []
    try:
        for k, nc in enumerate((1, 3, 5, 8)):
            p = str(tmp_path / f"c{nc}.mol")
            hg.molecules.write_alkane(p, nc)
            monkeypatch.setenv("H2G_TILE_ROWS", "256" if k % 2 else "512")
            h = hg.H2ERI.from_mol(p, qr_tol=1e-6)
            h.set_precision(hg.MIXED)
            hs.append(h)
        n = len(hs)
        dens = [np.stack([hg.molecules.seeded_density(h.num_bf, 2 + k, 950 + 10 * k + i) for i in range(2)])
                for k, h in enumerate(hs)]
        dDs = [torch.tensor(D, device="cuda") for D in dens]
        harr = (ctypes.c_void_p * n)(*[h.handle.value for h in hs])
        narr = (ctypes.c_int * n)(*([2] * n))
        darr = (ctypes.c_void_p * n)(*[t.data_ptr() for t in dDs])
        s = torch.cuda.current_stream()
        out = {}
        for mode in ("1", "0"):
            monkeypatch.setenv("H2G_BATCH_MERGED", mode)
            dJs = [torch.full_like(t, float("nan")) for t in dDs]
            jarr = (ctypes.c_void_p * n)(*[t.data_ptr() for t in dJs])
            rc = library.H2ERI_build_Coulomb_batch(n, harr, narr, darr, jarr, ctypes.c_void_p(s.cuda_stream))
            assert rc == 0, library.H2ERI_gpu_last_error()
            torch.cuda.synchronize()
            out[mode] = [t.cpu().numpy() for t in dJs]
        assert all(library.H2ERI_gpu_check(h.handle) == 0 for h in hs)
        for k, h in enumerate(hs):
            for i in range(2):
                assert relerr(out["1"][k][i], oracle_J(oracle_lib, h, dens[k][i])) < TOL_MIXED, (k, i)
                assert relerr(out["1"][k][i], out["0"][k][i]) < 1e-12, (k, i)
    finally:
        for h in hs:
            h.destroy()


@pytest.mark.parametrize("rows", ["512", "128", "0"])
def test_persistent_launch_against_range_launches(oracle_lib, library, monkeypatch, rows):
    """The whole mixed single-density matvec in one persistent launch (items
    taken from one work list, ranges waiting for the ranges they depend on)
    gives the J of the launch-per-range path up to the order of the FP64
    output sums, and both meet the 1e-8 target against the oracle; also with
    three densities per call on the single-density kernels, and with
    128-row tiles and tile heights chosen per range (0)."""
    torch = pytest.importorskip("torch")
    mol = os.path.join(GOLDEN, "alk32_ccpvdz.mol")
    monkeypatch.setenv("H2G_MMA_MIN_VEC", "17")   # several densities on the single-density kernels
    monkeypatch.setenv("H2G_TILE_ROWS", rows)
    out = {}
    for persist in ("1", "0"):
        monkeypatch.setenv("H2G_PERSIST", persist)
        h = hg.H2ERI.from_mol(mol, qr_tol=1e-6)
        try:
            h.set_precision(hg.MIXED)
            n = h.num_bf
            Ds = np.stack([hg.molecules.seeded_density(n, 41, 800 + i) for i in range(3)])
            dD = torch.tensor(Ds, device="cuda")
            dJ = torch.empty_like(dD)
            s = torch.cuda.Stream()
            torch.cuda.synchronize()
            for nd in (1, 3):
                assert library.H2ERI_build_Coulomb_device(h.handle, nd, dD.data_ptr(), dJ.data_ptr(),
                                                          ctypes.c_void_p(s.cuda_stream)) == 0
                s.synchronize()
                assert library.H2ERI_gpu_check(h.handle) == 0
                out[(persist, nd)] = dJ[:nd].cpu().numpy().copy()
            rep = h.report()
            assert rep["persist"] == int(persist)
            assert rep["tile_rows"] == int(rows)
            if persist == "1":
                assert rep["launches_per_matvec"] == 1 and rep["px_items"] > 0 and rep["px_grid"] > 0
            Jo = [oracle_J(oracle_lib, h, Ds[i]) for i in range(3)]
        finally:
            h.destroy()
        for nd in (1, 3):
            for i in range(nd):
                assert relerr(out[(persist, nd)][i], Jo[i]) < TOL_MIXED, (persist, nd, i)
    for nd in (1, 3):
        assert relerr(out[("1", nd)], out[("0", nd)]) < 1e-13


def test_drop_fp64_copy(oracle_lib, library, tmp_path):
    """H2ERI_gpu_drop_fp64: a structure in the mixed mode keeps giving the
    same J after its FP64 copy is freed, the device's free memory grows by
    about that copy, the FP64 mode is refused until the structure is
    released and uploaded again, and then FP64 J matches the oracle."""
    torch = pytest.importorskip("torch")
    p = str(tmp_path / "c6.mol")
    hg.molecules.write_alkane(p, 6)
    h = hg.H2ERI.from_mol(p, qr_tol=1e-6)
    try:
        D = hg.molecules.seeded_density(h.num_bf, 20, 77)
        Jo = np.zeros_like(D)
        oracle_lib.oracle_build_Coulomb(h.handle, D.ctypes.data, Jo.ctypes.data)
        assert library.H2ERI_gpu_drop_fp64(h.handle) == 3          # FP64 mode: refused
        h.set_precision(hg.MIXED)
        J1 = h.build_coulomb(D)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        assert library.H2ERI_gpu_drop_fp64(h.handle) == 0
        free1 = torch.cuda.mem_get_info()[0]
        arena = h.report()["arena_U"] + h.report()["arena_B"] + h.report()["arena_D"]
        assert free1 - free0 >= 0.9 * arena, (free1 - free0, arena)
        assert library.H2ERI_gpu_drop_fp64(h.handle) == 0          # idempotent
        J2 = h.build_coulomb(D)
        assert relerr(J2, J1) < 1e-14 and relerr(J2, Jo) < 1e-8
        assert library.H2ERI_gpu_set_precision(h.handle, hg.FP64) == 3
        assert b"dropped" in library.H2ERI_gpu_last_error()
        library.H2ERI_gpu_release(h.handle)
        h.set_precision(hg.FP64)
        assert relerr(h.build_coulomb(D), Jo) < 1e-12
    finally:
        h.destroy()
