"""Shared fixtures. Tests marked `gpu` need a CUDA device and call the GPU
library through its C ABI; everything else runs on the CPU (no compute calls
into the GPU library)."""
import ctypes
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "h2p-eri_gb300"))
sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")

import h2eri_gb300 as hg  # noqa: E402
from h2eri_gb300 import build as hg_build  # noqa: E402
from h2eri_gb300 import molecules  # noqa: E402
from oracle import build_oracle  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the C ABI of libh2eri_gb300.so")
    config.addinivalue_line("markers", "slow: takes more than ~30 s on 8 cores")


@pytest.fixture(scope="session")
def library():
    hg_build.build()
    return hg.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    path = build_oracle.build()
    L = ctypes.CDLL(path)
    for f in ("oracle_matvec", "oracle_build_Coulomb", "oracle_build_exchange"):
        if hasattr(L, f):
            getattr(L, f).argtypes = [ctypes.c_void_p] * 3
            getattr(L, f).restype = None
    return L


def ref_lib_or_skip():
    """The reference compiled from its own sources (only where they exist)."""
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("reference sources not present on this machine")
    path = build_ref.build(verbose=False)
    L = ctypes.CDLL(path)
    for f in ("H2ERI_matvec", "H2ERI_build_Coulomb", "H2ERI_build_exchange"):
        getattr(L, f).argtypes = [ctypes.c_void_p] * 3
        getattr(L, f).restype = None
    for f in ("H2ERI_exchange_workbuf_init", "H2ERI_exchange_workbuf_free"):
        getattr(L, f).argtypes = [ctypes.c_void_p]
        getattr(L, f).restype = None
    L.oref_build.restype = ctypes.c_void_p
    L.oref_build.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    L.oref_struct_size.restype = ctypes.c_size_t
    return L


def golden(name, n=None):
    a = np.fromfile(os.path.join(GOLDEN, name))
    return a.reshape(n, n) if n else a


@pytest.fixture(scope="session")
def alk32(library):
    """C10H22 (alk32_ccpvdz.mol of the reference tests), QR tol 1e-6."""
    h = hg.H2ERI.from_mol(os.path.join(GOLDEN, "alk32_ccpvdz.mol"), qr_tol=1e-6)
    yield h
    h.destroy()


@pytest.fixture(scope="session")
def alk26(library):
    """C8H18 (alk26_ccpvdz.mol of the reference tests), QR tol 1e-6."""
    h = hg.H2ERI.from_mol(os.path.join(GOLDEN, "alk26_ccpvdz.mol"), qr_tol=1e-6)
    yield h
    h.destroy()


@pytest.fixture(scope="session")
def small_mols(library, tmp_path_factory):
    """Edge-case molecules: one atom (single leaf, no far field), ethane
    (single level), butane (first admissible pairs)."""
    d = tmp_path_factory.mktemp("mols")
    out = {}
    for name, n in (("CH4", 1), ("C2H6", 2), ("C4H10", 4)):
        p = str(d / f"{name}.mol")
        molecules.write_alkane(p, n)
        out[name] = hg.H2ERI.from_mol(p, qr_tol=1e-6)
    yield out
    for h in out.values():
        h.destroy()


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))
