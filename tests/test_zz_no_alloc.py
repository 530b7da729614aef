"""H2ERI_matvec_device_noalloc: the matvec for callers that must not allocate
device memory after set-up (a fixed device-memory budget, a memory pool owned
by the host application, or loops where cudaMalloc/cudaFree would
synchronise the device). It uses a fixed 16 MiB device array for its
intermediates. Checked through the C ABI against H2ERI_matvec_device on two
calls in a row (the array keeps the previous call's contents, so the second
call also shows that it is cleared), to the FP64 tolerance of the other GPU
tests. This file sorts last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import relerr

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-12


def test_noalloc_matches_device_entry_point(alk26, library):
    torch = pytest.importorskip("torch")
    alk26.set_precision(hg.FP64)
    alk26.upload()
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    rng = np.random.default_rng(2024)
    for call in range(2):
        x = torch.tensor(rng.standard_normal(alk26.krnl_mat_size), device="cuda")
        y_ref = torch.empty_like(x)
        y = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        assert library.H2ERI_matvec_device(alk26.handle, 1, x.data_ptr(), y_ref.data_ptr(), sp) == 0
        rc = library.H2ERI_matvec_device_noalloc(alk26.handle, x.data_ptr(), y.data_ptr(), sp)
        assert rc == 0, library.H2ERI_gpu_last_error()
        s.synchronize()
        e = relerr(y.cpu().numpy(), y_ref.cpu().numpy())
        assert e < TOL_FP64, (call, e)


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
