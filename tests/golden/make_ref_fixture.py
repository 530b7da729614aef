"""Writes a fixture produced by the reference itself: an H2 representation
built by the reference's own set-up (H2ERI_init / CMS_read_mol_file /
H2ERI_process_shells / H2ERI_partition / H2ERI_build_H2 at QR tolerance
1e-6, compiled from its sources by oracle/build_ref.py), saved in this
package's representation format, together with the reference's own results
on it.

The system is a linear chain of 40 hydrogen atoms 2.0 Angstrom apart
(cc-pVDZ, s and p shells, 200 Cartesian basis functions). A C4H10 built the
same way takes 57 MB (its near-field blocks alone hold 6.7 M doubles); the
chain's tree has 15 nodes, 12 admissible and 7 inadmissible pairs and takes
9 MB, so the fixture covers the upward sweep, coupling blocks, downward
sweep and near field at a size that can be committed.

  ref_h40.h2r        the representation (H2ERI_save_representation reads the
                     struct fields only; the struct layout is the reference's)
  ref_h40_x.bin      a seeded vector of krnl_mat_size doubles (seed 5149)
  ref_h40_y.bin      the reference's H2ERI_matvec of it
  ref_h40_D.bin      a seeded density (200 x 200, n_occ 20, seed 5150)
  ref_h40_J.bin      the reference's H2ERI_build_Coulomb of it
  ref_h40_K.bin      the reference's H2ERI_build_exchange of it

The GPU tests load the representation and compare their results with these
numbers directly, so the FP64 claim against the reference does not pass
through the oracle. Run where the reference sources exist:
python tests/golden/make_ref_fixture.py
"""
import ctypes
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "h2p-eri_gb300"))
sys.path.insert(0, REPO)

import h2eri_gb300 as hg  # noqa: E402
from h2eri_gb300 import build as hb, molecules  # noqa: E402
from oracle import build_ref  # noqa: E402

QR_TOL = 1e-6
N_ATOM, SPACING = 40, 2.0
X_SEED, D_SEED, N_OCC = 5149, 5150, 20


def main():
    if not build_ref.available():
        raise SystemExit("reference sources absent: the fixture can only be made where they exist")
    hb.build()
    L = hg.lib()
    R = ctypes.CDLL(build_ref.build(verbose=False))
    R.oref_build.restype = ctypes.c_void_p
    R.oref_build.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    for f in ("H2ERI_matvec", "H2ERI_build_Coulomb", "H2ERI_build_exchange"):
        getattr(R, f).argtypes = [ctypes.c_void_p] * 3
        getattr(R, f).restype = None
    with tempfile.TemporaryDirectory() as d:
        mol = os.path.join(d, "h40.mol")
        xyz = np.array([[i * SPACING, 0.0, 0.0] for i in range(N_ATOM)])
        molecules.write_mol(mol, ["H"] * N_ATOM, xyz)
        rh = R.oref_build(mol.encode(), 1e-10, 1e-10, QR_TOL, 0)
    s = ctypes.cast(rh, ctypes.POINTER(hg.H2ERIStruct)).contents
    krnl, nbf = s.krnl_mat_size, s.num_bf
    rc = L.H2ERI_save_representation(ctypes.c_void_p(rh), os.path.join(HERE, "ref_h40.h2r").encode())
    assert rc == 0, rc
    x = np.random.default_rng(X_SEED).standard_normal(krnl)
    y = np.zeros_like(x)
    R.H2ERI_matvec(rh, x.ctypes.data, y.ctypes.data)
    D = molecules.seeded_density(nbf, N_OCC, D_SEED)
    J = np.zeros_like(D)
    K = np.zeros_like(D)
    R.H2ERI_build_Coulomb(rh, D.ctypes.data, J.ctypes.data)
    R.H2ERI_build_exchange(rh, D.ctypes.data, K.ctypes.data)
    for name, a in (("x", x), ("y", y), ("D", D), ("J", J), ("K", K)):
        a.tofile(os.path.join(HERE, f"ref_h40_{name}.bin"))
    print(f"H40: {nbf} bf, krnl_mat_size {krnl}, {s.n_r_adm_pair} admissible / {s.n_r_inadm_pair} inadmissible "
          f"pairs, |y| {np.linalg.norm(y):.6e}, |J| {np.linalg.norm(J):.6e}, |K| {np.linalg.norm(K):.6e}")


if __name__ == "__main__":
    main()
