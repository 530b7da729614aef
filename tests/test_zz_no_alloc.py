"""H2ERI_matvec_device_noalloc: the matvec for callers that must not allocate
device memory after set-up (a fixed device-memory budget, a memory pool owned
by the host application, or loops where cudaMalloc/cudaFree would
synchronise the device). It uses a fixed 16 MiB device array for its
intermediates. Checked through the C ABI against the FP64 oracle and against
H2ERI_matvec_device on two calls in a row (the array keeps the previous
call's contents, so the second call also shows that it is cleared), to the
FP64 tolerance of the other GPU tests; that a call leaves the device's free
memory unchanged; and its argument checks. This file sorts last so that a
run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import relerr

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def test_noalloc_matches_oracle_and_device_entry_point(alk26, library, oracle_lib):
    torch = pytest.importorskip("torch")
    alk26.set_precision(hg.FP64)
    alk26.upload()
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    rng = np.random.default_rng(2024)
    for call in range(2):
        xh = rng.standard_normal(alk26.krnl_mat_size)
        x = torch.tensor(xh, device="cuda")
        y_ref = torch.empty_like(x)
        y = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        assert library.H2ERI_matvec_device(alk26.handle, 1, x.data_ptr(), y_ref.data_ptr(), sp) == 0
        rc = library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), sp)
        assert rc == 0, library.H2ERI_gpu_last_error()
        s.synchronize()
        assert library.H2ERI_gpu_check(alk26.handle) == 0
        yo = np.zeros_like(xh)
        oracle_lib.oracle_matvec(alk26.handle, xh.ctypes.data, yo.ctypes.data)
        e_o = relerr(y.cpu().numpy(), yo)
        e_d = relerr(y.cpu().numpy(), y_ref.cpu().numpy())
        assert e_o < TOL_FP64, (call, e_o)
        assert e_d < TOL_FP64, (call, e_d)


def test_noalloc_leaves_free_memory_unchanged(alk26, library):
    torch = pytest.importorskip("torch")
    alk26.set_precision(hg.FP64)
    alk26.upload()
    x = torch.tensor(np.random.default_rng(7).standard_normal(alk26.krnl_mat_size), device="cuda")
    y = torch.empty_like(x)
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    assert library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), sp) == 0   # warm-up
    s.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), sp) == 0
    s.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_argument_checks(alk26, library, monkeypatch):
    """Null vectors (status 3) and a representation whose scratch need is
    above the limit (status 4; the limit is lowered through the environment
    to just below this structure's need, as reported by H2ERI_gpu_report)."""
    torch = pytest.importorskip("torch")
    alk26.upload()
    x = torch.zeros(alk26.krnl_mat_size, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    assert library.H2ERI_matvec_device_noalloc(alk26.handle, None, y.data_ptr(), None) == 3
    assert library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), None, None) == 3
    assert b"null" in library.H2ERI_gpu_last_error()
    need = int(alk26.report()["noalloc_scratch_doubles"])
    assert 0 < need <= 1 << 21
    monkeypatch.setenv("H2G_NOALLOC_LIMIT", str(need - 1))
    assert library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), None) == 4
    assert str(need).encode() in library.H2ERI_gpu_last_error()
    monkeypatch.setenv("H2G_NOALLOC_LIMIT", str(need))
    assert library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), None) == 0
    monkeypatch.setenv("H2G_NOALLOC_LIMIT", str(1 << 40))   # cannot raise the limit above the array
    assert library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert library.H2ERI_gpu_check(alk26.handle) == 0


def test_noalloc_requires_upload(library, tmp_path):
    """A structure that was never uploaded is rejected (no implicit upload,
    which would allocate)."""
    torch = pytest.importorskip("torch")
    mol = str(tmp_path / "ch4.mol")
    hg.molecules.write_alkane(mol, 1)
    h = hg.H2ERI.from_mol(mol, qr_tol=1e-6)
    try:
        x = torch.zeros(h.krnl_mat_size, dtype=torch.float64, device="cuda")
        y = torch.zeros_like(x)
        rc = library.H2ERI_matvec_device_noalloc(h.handle, x.data_ptr(), y.data_ptr(), None)
        assert rc != 0
        assert b"H2ERI_gpu_upload" in library.H2ERI_gpu_last_error()
    finally:
        h.destroy()
