"""The host set-up (mol reader, shell processing, partition, H2
construction with its pivoted QR and integral engine, representation save
and load) built from its sources with AddressSanitizer and
UndefinedBehaviorSanitizer and run on C4H10 with OpenMP threads: no
out-of-bounds access, use after free or undefined behaviour is reported."""
import os
import shutil
import subprocess

import pytest

from h2eri_gb300 import molecules

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(REPO, "h2p-eri_gb300", "csrc", "host")
GPU = os.path.join(REPO, "h2p-eri_gb300", "csrc", "gpu")


def test_host_setup_under_sanitizers(tmp_path):
    if shutil.which("g++") is None or shutil.which("gcc") is None:
        pytest.skip("no host compiler")
    san = ["-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=all",
           "-fopenmp", "-ffp-contract=off"]
    inc = ["-I" + HOST, "-I" + GPU, "-I" + os.path.join(REPO, "include")]
    ints = str(tmp_path / "ints.o")
    subprocess.run(["gcc", "-std=gnu11", "-c", os.path.join(HOST, "h2g_ints.c"), "-o", ints] + san + inc,
                   check=True, capture_output=True, timeout=300)
    exe = str(tmp_path / "setup_san")
    srcs = [os.path.join(REPO, "tests", "sanitize_setup_main.cpp")] + \
        [os.path.join(HOST, f) for f in ("h2g_build.cpp", "h2g_setup.cpp", "h2g_io.cpp")]
    subprocess.run(["g++", "-std=c++17", "-o", exe] + srcs + [ints] + san + inc,
                   check=True, capture_output=True, timeout=300)
    mol = str(tmp_path / "c4.mol")
    molecules.write_alkane(mol, 4)
    env = dict(os.environ, OMP_NUM_THREADS="4", ASAN_OPTIONS="detect_leaks=0:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, mol, "1e-6", str(tmp_path / "c4.h2r")], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-4000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-4000:]
    assert "num_bf" in r.stdout
