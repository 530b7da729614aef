"""The .mol reader (CMS_read_mol_file, H2P-ERI src/CMS.c:14-123) on
malformed input: it stops the process with a message instead of reading past
the error (the reference's reader has no checks). Each case runs in a child
process because the failure aborts."""
import os
import subprocess
import sys

import pytest

# case: (file content or None for a missing file, expected message)
BAD_MOL = {
    "missing": (None, "cannot open mol file"),
    "negative atom count": ("-2\n", "bad mol header"),
    "truncated coordinates": ("1\nH 1 3 3\n0.0 0.0\n", "bad coordinates"),
    "unknown shell type": ("1\nH 1 1 1\n0.0 0.0 0.0\nQ 1 1\n1.0 1.0\n", "unknown shell type"),
    "no primitives": ("1\nH 1 0 0\n0.0 0.0 0.0\nS 0 1\n", "bad shell header"),
    "missing coefficient": ("1\nH 1 2 2\n0.0 0.0 0.0\nS 2 1\n1.0 0.5\n0.3\n", "bad coefficient"),
}


@pytest.mark.parametrize("case", sorted(BAD_MOL))
def test_malformed_mol_file_fails_loudly(library, tmp_path, case):
    text, message = BAD_MOL[case]
    path = tmp_path / "bad.mol"
    if text is not None:
        path.write_text(text)
    code = ("import ctypes, sys; import h2eri_gb300 as hg; L = hg.lib(); "
            "n = ctypes.c_int(); s = ctypes.c_int(); p = ctypes.c_void_p(); "
            "L.CMS_read_mol_file(sys.argv[1].encode(), ctypes.byref(n), ctypes.byref(s), ctypes.byref(p))")
    r = subprocess.run([sys.executable, "-c", code, str(path)], capture_output=True, text=True, timeout=120,
                       cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       env=dict(os.environ, PYTHONPATH=os.pathsep.join(sys.path)))
    assert r.returncode != 0
    assert message in r.stderr, r.stderr
