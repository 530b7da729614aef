"""The C ABI library loads without a GPU and exports every function that
include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import REPO

DECL = re.compile(r"^\s*(?:void|int|const char \*|double|size_t)\s+\*?\s*(\w+)\s*\(", re.M)


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names.update(DECL.findall(src))
    return sorted(names)


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for f in ("H2ERI_init", "H2ERI_destroy", "H2ERI_print_statistic", "H2ERI_process_shells", "H2ERI_partition",
              "H2ERI_build_H2", "H2ERI_matvec", "H2ERI_build_Coulomb", "H2ERI_build_exchange",
              "H2ERI_exchange_workbuf_init", "H2ERI_exchange_workbuf_free", "CMS_read_mol_file"):
        assert f in names, f


def test_library_exports_every_declared_symbol(library):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(library, n)]
    assert not missing, missing


def test_library_loads_without_gpu_and_reports_errors(library):
    # a null handle is rejected with a message, not a crash
    rc = library.H2ERI_gpu_upload(None)
    assert rc != 0
    assert library.H2ERI_gpu_last_error()


@pytest.mark.parametrize("device_bytes", [100e9, 2e6])
def test_exchange_plan_in_bounds(small_mols, alk26, library, device_bytes):
    """The exchange plan (built on the host, no GPU) keeps every access of
    every planned kernel inside its buffer, with one or many n ranges."""
    for h in list(small_mols.values()) + [alk26]:
        out = np.zeros(5)
        rc = library.H2ERI_exchange_plan_check(h.handle, device_bytes, out.ctypes.data, 5)
        assert rc == 0, library.H2ERI_gpu_last_error()
        assert out[0] > 0 and out[1] >= 1 and out[4] > 0


def test_exchange_plan_in_bounds_3d_cluster(library, tmp_path):
    """The same on a 3-D system (8 CH4 on a jittered lattice: every node has
    neighbours on all sides), with the work tensors in one range, a few and
    many ranges of n."""
    import h2eri_gb300 as hg
    p = str(tmp_path / "ch4x8.mol")
    hg.molecules.write_methane_cluster(p, shape=(2, 2, 2))
    h = hg.H2ERI.from_mol(p, qr_tol=1e-7)
    try:
        ranges = []
        for device_bytes in (100e9, 2e8, 2e6):
            out = np.zeros(5)
            rc = library.H2ERI_exchange_plan_check(h.handle, device_bytes, out.ctypes.data, 5)
            assert rc == 0, library.H2ERI_gpu_last_error()
            assert out[0] > 0 and out[4] > 0
            ranges.append(out[1])
        assert ranges[0] == 1 and ranges[2] > ranges[1] > 1
    finally:
        h.destroy()
