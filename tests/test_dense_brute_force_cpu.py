"""Independent check of the whole J/K chain against brute force: the full
ERI tensor of a small molecule, from the same shells through the integral
engine, contracted with a density exactly, against the J and K of the H2
representation (computed by the oracle, the CPU restatement of the
reference, on the representation the GPU uses). CH4 is one leaf; C2H6 has
nine nodes but no admissible pair, so at QR tolerance 1e-10 both H2 matrices
equal the dense tensor up to rounding (measured ~1e-15), and at QR tolerance
1e-6 C2H6's compressed near-field blocks give errors at that level (measured
2.8e-7 on J, 1.3e-6 on K). The far field (coupling blocks, which start at
C4H10, whose dense tensor would take 1.2 GB) is pinned instead by the oracle
against the reference and the reference's golden J and K. Also: J is
symmetric, the Coulomb energy tr(D J) of a projector density is positive and
the ERI matrix over basis-function pairs is positive semi-definite."""
import ctypes

import numpy as np
import pytest

import h2eri_gb300 as hg
from h2eri_gb300 import molecules
from conftest import relerr


class ShellT(ctypes.Structure):
    """struct simint_shell (include/h2eri_types.h)."""
    _fields_ = [("am", ctypes.c_int), ("nprim", ctypes.c_int), ("x", ctypes.c_double), ("y", ctypes.c_double),
                ("z", ctypes.c_double), ("alpha", ctypes.POINTER(ctypes.c_double)),
                ("coef", ctypes.POINTER(ctypes.c_double)), ("memsize", ctypes.c_size_t),
                ("ptr", ctypes.c_void_p)]


class Pair(ctypes.Structure):
    _fields_ = [("am1", ctypes.c_int), ("am2", ctypes.c_int), ("nprim", ctypes.c_int),
                ("A", ctypes.c_double * 3), ("B", ctypes.c_double * 3)] + \
               [(n, ctypes.POINTER(ctypes.c_double)) for n in ("P", "p", "K", "ip")]


def ncart(l):
    return (l + 1) * (l + 2) // 2


def dense_eri(library, h):
    """(mn|pq) over all basis functions, 8-fold symmetric fill."""
    library.h2g_ints_init()
    library.h2g_pair_init.argtypes = [ctypes.POINTER(Pair), ctypes.POINTER(ShellT), ctypes.POINTER(ShellT)]
    library.h2g_eri_quartet.argtypes = [ctypes.POINTER(Pair), ctypes.POINTER(Pair), ctypes.c_void_p]
    s = h.s
    nsh, nbf = s.nshell, s.num_bf
    sh = ctypes.cast(s.shells, ctypes.POINTER(ShellT))
    sb = np.ctypeslib.as_array(s.shell_bf_sidx, shape=(nsh + 1,)).copy()
    pairs = {}
    for i in range(nsh):
        for j in range(i + 1):
            p = Pair()
            library.h2g_pair_init(ctypes.byref(p), ctypes.byref(sh[i]), ctypes.byref(sh[j]))
            pairs[i, j] = p
    G = np.zeros((nbf, nbf, nbf, nbf))
    ij = [(i, j) for i in range(nsh) for j in range(i + 1)]
    for a, (i, j) in enumerate(ij):
        for (k, l) in ij[:a + 1]:
            n = [ncart(sh[x].am) for x in (i, j, k, l)]
            out = np.zeros(int(np.prod(n)))
            library.h2g_eri_quartet(ctypes.byref(pairs[i, j]), ctypes.byref(pairs[k, l]), out.ctypes.data)
            blk = out.reshape(n)
            si, sj, sk, sl = (slice(sb[x], sb[x + 1]) for x in (i, j, k, l))
            for (A, B, C, D), t in (((si, sj, sk, sl), (0, 1, 2, 3)), ((sj, si, sk, sl), (1, 0, 2, 3)),
                                    ((si, sj, sl, sk), (0, 1, 3, 2)), ((sj, si, sl, sk), (1, 0, 3, 2))):
                v = blk.transpose(t)
                G[A, B, C, D] = v
                G[C, D, A, B] = v.transpose(2, 3, 0, 1)
    return G


def oracle_JK(oracle_lib, h, D):
    J, K = np.zeros_like(D), np.zeros_like(D)
    oracle_lib.oracle_build_Coulomb(h.handle, D.ctypes.data, J.ctypes.data)
    oracle_lib.oracle_build_exchange(h.handle, D.ctypes.data, K.ctypes.data)
    return J, K


@pytest.mark.parametrize("n_carbon,qr_tol,tol", [(1, 1e-10, 1e-12), (2, 1e-10, 1e-12), (2, 1e-6, 1e-5)])
def test_h2_J_K_against_dense_eri(library, oracle_lib, tmp_path, n_carbon, qr_tol, tol):
    p = str(tmp_path / f"c{n_carbon}.mol")
    molecules.write_alkane(p, n_carbon)
    h = hg.H2ERI.from_mol(p, qr_tol=qr_tol)
    try:
        G = dense_eri(library, h)
        nbf = h.num_bf
        D = molecules.seeded_density(nbf, 2 * n_carbon + 1, 5150 + n_carbon)
        J_dense = np.einsum("mnpq,pq->mn", G, D)
        K_dense = np.einsum("mnpq,np->mq", G, D)
        J, K = oracle_JK(oracle_lib, h, D)
        assert relerr(J, J_dense) < tol
        assert relerr(K, K_dense) < tol
        np.testing.assert_allclose(J, J.T, rtol=0, atol=1e-12 * np.abs(J).max())
        assert float(np.sum(D * J)) > 0.0
        # the ERI matrix over basis-function pairs is positive semi-definite
        w = np.linalg.eigvalsh(G.reshape(nbf * nbf, nbf * nbf))
        assert w.min() > -1e-10 * w.max()
    finally:
        h.destroy()
