"""The autotuner (H2ERI_gpu_autotune): every candidate launch configuration
is timed on the device and the fastest kept. Whatever it picks (tile rows
512 / 256 / 128 rebuild the single-density plan; tiles per CTA; near-field
lanes; tensor-core kernel or not for several densities), J must stay at the
oracle's to the tolerance of the precision; the choice is reported, cached
by structure shape and, through H2G_TUNE_FILE, read back by another
process."""
import os
import subprocess
import sys

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import REPO, relerr

pytestmark = pytest.mark.gpu


def oracle_J(oracle_lib, h, D):
    J = np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(h.handle, np.ascontiguousarray(D).ctypes.data, J.ctypes.data)
    return J


@pytest.mark.parametrize("mode,tol", [(hg.FP64, 1e-12), (hg.MIXED, 1e-8)])
def test_autotune_single_density(alk26, oracle_lib, mode, tol):
    alk26.set_precision(mode)
    try:
        r = alk26.autotune(1)
        assert r["candidates"] >= 6 and r["ms_best"] <= r["ms_before"] * 1.0001
        assert r["choice"]["tile_rows"] in (0, 128, 256, 512)   # 0: chosen per range
        rep = alk26.report()
        assert rep["tile_rows"] == r["choice"]["tile_rows"]
        D = hg.molecules.seeded_density(alk26.num_bf, 30, 6100 + mode)
        assert relerr(alk26.build_coulomb(D), oracle_J(oracle_lib, alk26, D)) < tol
    finally:
        alk26.set_precision(hg.FP64)


@pytest.mark.parametrize("rows,tpc", [(0, 2), (128, 1), (256, 2), (512, 1)])
def test_tile_shapes_the_tuner_may_pick(oracle_lib, tmp_path, monkeypatch, rows, tpc):
    """Every tile shape among the tuner's candidates, fixed through the
    environment, gives the oracle's J in both precisions."""
    monkeypatch.setenv("H2G_TILE_ROWS", str(rows))
    monkeypatch.setenv("H2G_TILES_PER_CTA", str(tpc))
    p = str(tmp_path / "c6.mol")
    hg.molecules.write_alkane(p, 6)
    h = hg.H2ERI.from_mol(p, qr_tol=1e-6)
    try:
        D = hg.molecules.seeded_density(h.num_bf, 20, 6300 + rows)
        Jo = oracle_J(oracle_lib, h, D)
        assert relerr(h.build_coulomb(D), Jo) < 1e-12
        assert h.report()["tile_rows"] == rows
        h.set_precision(hg.MIXED)
        assert relerr(h.build_coulomb(D), Jo) < 1e-8
        assert h.report()["tiles_per_cta"] == tpc
    finally:
        h.destroy()


def test_autotune_multi_density(alk32, oracle_lib):
    alk32.set_precision(hg.MIXED)
    try:
        r = alk32.autotune(16)
        assert r["candidates"] >= 10
        Ds = np.stack([hg.molecules.seeded_density(alk32.num_bf, 41, 6200 + i) for i in range(16)])
        J = alk32.build_coulomb(Ds)
        for i in (0, 7, 15):
            assert relerr(J[i], oracle_J(oracle_lib, alk32, Ds[i])) < 1e-8
        r2 = alk32.autotune(2)
        J2 = alk32.build_coulomb(Ds[:2])
        for i in range(2):
            assert relerr(J2[i], oracle_J(oracle_lib, alk32, Ds[i])) < 1e-8
        print("tuned:", r["choice"], r["ms_before"], "->", r["ms_best"], "| 2 densities:", r2["choice"])
    finally:
        alk32.set_precision(hg.FP64)


_CHILD = r"""
import sys, os
sys.path.insert(0, os.path.join({repo!r}, "h2p-eri_gb300"))
import h2eri_gb300 as hg
hg.molecules.write_alkane({mol!r}, 4)
h = hg.H2ERI.from_mol({mol!r}, qr_tol=1e-6)
h.set_precision(hg.MIXED)
if sys.argv[1] == "tune":
    r = h.autotune(1)
    print(r["choice"]["tile_rows"], r["choice"]["tiles_per_cta"], r["choice"]["nf_concurrent"])
else:
    rep = h.report()
    print(int(rep["tile_rows"]), int(rep["tiles_per_cta"]), int(rep["nf_concurrent"]))
h.destroy()
"""


def test_tuning_file_read_by_another_process(tmp_path):
    tune = str(tmp_path / "tune.txt")
    script = _CHILD.format(repo=REPO, mol=str(tmp_path / "c4h10.mol"))
    env = dict(os.environ, H2G_TUNE_FILE=tune)
    a = subprocess.run([sys.executable, "-c", script, "tune"], env=env, capture_output=True, text=True, timeout=600)
    assert a.returncode == 0, a.stderr[-2000:]
    assert os.path.getsize(tune) > 0
    b = subprocess.run([sys.executable, "-c", script, "read"], env=env, capture_output=True, text=True, timeout=600)
    assert b.returncode == 0, b.stderr[-2000:]
    assert a.stdout.split() == b.stdout.split()
