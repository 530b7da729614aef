"""Set-up on the GPU: the dense near-field (D) and full coupling (B) blocks
of electron-repulsion integrals evaluated by the GPU engine (h2g_eri.cu)
equal the host engine's to 1e-13 of the largest value (same recurrences and
tables; only the order of sums differs); so do the sketched matrices of the
nested-basis construction (proxy-point potentials and far-field ERIs times
their sparse sign sketches); and a representation built with the GPU
integrals gives the oracle's J to 1e-12 on itself and the reference's golden
J to the H2 tolerance, as the host-built one does."""
import ctypes
import os
import time

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, relerr

pytestmark = pytest.mark.gpu


def eri_check(library, h, max_blocks):
    out = np.zeros(6)
    rc = library.H2ERI_gpu_setup_eri_check(h.handle, max_blocks, out.ctypes.data)
    assert rc == 0, library.H2ERI_gpu_last_error()
    return out


@pytest.mark.parametrize("name", ["CH4", "C2H6", "C4H10"])
def test_gpu_blocks_equal_host_engine_small(small_mols, library, name):
    dmax, vmax, n, nb = eri_check(library, small_mols[name], 1000)[:4]
    assert nb >= 1 and n > 0
    assert dmax <= 1e-13 * vmax, (dmax, vmax)


def test_gpu_blocks_equal_host_engine_alk32(alk32, library):
    """Every class of (s, p, d) quartets of C10H22 occurs in these blocks."""
    dmax, vmax, n, nb, t_gpu, t_host = eri_check(library, alk32, 40)
    assert nb >= 40 and n > 1e6
    assert dmax <= 1e-13 * vmax, (dmax, vmax)
    print(f"C10H22 {int(nb)} blocks, {n / 1e6:.1f} M integrals: GPU {t_gpu:.3f} s, host engine (one thread) "
          f"{t_host:.3f} s")


def u_check(library, h, max_nodes):
    out = np.zeros(6)
    rc = library.H2ERI_gpu_setup_u_check(h.handle, max_nodes, out.ctypes.data)
    assert rc == 0, library.H2ERI_gpu_last_error()
    return out


@pytest.mark.parametrize("name", ["CH4", "C2H6", "C4H10"])
def test_gpu_nested_basis_matrices_equal_host_engine_small(small_mols, library, name):
    dmax, vmax, n, nn = u_check(library, small_mols[name], 1000)[:4]
    assert nn >= 1 and n > 0
    assert dmax <= 1e-13 * vmax, (dmax, vmax)


def test_gpu_nested_basis_matrices_equal_host_engine_alk32(alk32, library):
    """Leaf and upper-level nodes of C10H22: s, p and d pairs against
    proxy points and far-field pairs of every class."""
    dmax, vmax, n, nn, t_gpu, t_host = u_check(library, alk32, 1000)
    assert nn >= 8 and n > 1e5
    assert dmax <= 1e-13 * vmax, (dmax, vmax)
    print(f"C10H22 nested bases: {int(nn)} nodes, {n / 1e6:.2f} M sketched entries: GPU {t_gpu:.3f} s, host engine "
          f"(one thread) {t_host:.3f} s")


def test_representation_built_with_gpu_blocks(oracle_lib, library, monkeypatch):
    mol = os.path.join(GOLDEN, "alk32_ccpvdz.mol")
    times = {}
    hs = {}
    try:
        for flag in ("1", "0"):
            monkeypatch.setenv("H2G_SETUP_GPU", flag)
            t0 = time.perf_counter()
            hs[flag] = hg.H2ERI.from_mol(mol, qr_tol=1e-6)
            times[flag] = time.perf_counter() - t0
        n = hs["1"].num_bf
        D = np.fromfile(os.path.join(GOLDEN, "D_alk32_ccpvdz.bin")).reshape(n, n)
        Jg = np.fromfile(os.path.join(GOLDEN, "J_alk32_ccpvdz.bin")).reshape(n, n)
        J = {}
        for flag, h in hs.items():
            J[flag] = h.build_coulomb(D)
            Jo = np.zeros_like(D)
            oracle_lib.oracle_build_Coulomb(h.handle, D.ctypes.data, Jo.ctypes.data)
            assert relerr(J[flag], Jo) < 1e-12, flag
        # the golden J of the reference holds to the H2 tolerance for both
        e1, e0 = relerr(J["1"], Jg), relerr(J["0"], Jg)
        assert e1 < 2e-7 and e0 < 2e-7, (e1, e0)
        # same blocks up to rounding: the two representations agree far below
        # the H2 tolerance (pivots of the compression may differ on ties)
        assert relerr(J["1"], J["0"]) < 1e-7
        s1, s0 = hs["1"].s, hs["0"].s
        print(f"set-up C10H22: GPU blocks {times['1']:.2f} s, host blocks {times['0']:.2f} s; "
              f"B+D build {s1.timers[2] + s1.timers[3]:.2f} vs {s0.timers[2] + s0.timers[3]:.2f} s")
    finally:
        for h in hs.values():
            h.destroy()
