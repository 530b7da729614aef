"""Synthetic alkane generator used by the benchmark and the tests."""
import numpy as np

from h2eri_gb300 import molecules


def test_alkane_composition_and_geometry():
    for n in (1, 2, 10, 30):
        syms, xyz = molecules.alkane_coords(n)
        assert syms.count("C") == n and syms.count("H") == 2 * n + 2
        c = xyz[:n]
        h = xyz[n:]
        if n > 1:
            dcc = np.linalg.norm(np.diff(c, axis=0), axis=1)
            np.testing.assert_allclose(dcc, 1.54, atol=1e-12)
        # every H sits 1.09 A from its nearest carbon
        d = np.linalg.norm(h[:, None, :] - c[None, :, :], axis=2).min(axis=1)
        np.testing.assert_allclose(d, 1.09, atol=1e-12)
        # H-C-H and C-C-C angles are tetrahedral
        if n > 2:
            v1, v2 = c[0] - c[1], c[2] - c[1]
            ang = np.degrees(np.arccos(v1 @ v2 / np.linalg.norm(v1) / np.linalg.norm(v2)))
            assert abs(ang - 109.4712206) < 1e-6


def test_mol_file_round_trip(tmp_path):
    p = tmp_path / "c3.mol"
    molecules.write_alkane(str(p), 3)
    lines = p.read_text().split("\n")
    assert int(lines[0]) == 11
    assert lines[1].split()[0] == "C"


def test_seeded_density_is_projector():
    D = molecules.seeded_density(50, 7, seed=1000)
    np.testing.assert_allclose(D, D.T, atol=1e-14)
    np.testing.assert_allclose(D @ D, D, atol=1e-12)
    assert abs(np.trace(D) - 7) < 1e-12



def test_methane_cluster_geometry():
    """48 CH4 on a jittered 4 x 4 x 3 lattice: tetrahedral molecules with
    C-H 1.09 A, centres within the jitter of their sites, no two atoms of
    different molecules closer than 1.2 A, reproducible from the seed."""
    syms, xyz = molecules.methane_cluster_coords()
    assert syms.count("C") == 48 and syms.count("H") == 192
    c, h = xyz[:48], xyz[48:].reshape(48, 4, 3)
    for m in range(48):
        d = np.linalg.norm(h[m] - c[m], axis=1)
        np.testing.assert_allclose(d, 1.09, atol=1e-12)
        u = (h[m] - c[m]) / 1.09
        g = u @ u.T
        np.testing.assert_allclose(g[np.triu_indices(4, 1)], -1.0 / 3.0, atol=1e-12)
    sites = np.array([[i, j, k] for i in range(4) for j in range(4) for k in range(3)], dtype=float) * 4.0
    assert np.abs(c - sites).max() <= 0.2
    mol_of = np.repeat(np.arange(48), 1).tolist() + np.repeat(np.arange(48), 4).tolist()
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    other = np.array(mol_of)[:, None] != np.array(mol_of)[None, :]
    assert d[other].min() > 1.2
    syms2, xyz2 = molecules.methane_cluster_coords()
    np.testing.assert_array_equal(xyz, xyz2)


def test_methane_cluster_geometry():
    """48 CH4 on a jittered 4 x 4 x 3 lattice: tetrahedral molecules with
    C-H 1.09 A, centres within the jitter of their sites, no two atoms of
    different molecules closer than 1.2 A, reproducible from the seed."""
    syms, xyz = molecules.methane_cluster_coords()
    assert syms.count("C") == 48 and syms.count("H") == 192
    c, h = xyz[:48], xyz[48:].reshape(48, 4, 3)
    for m in range(48):
        d = np.linalg.norm(h[m] - c[m], axis=1)
        np.testing.assert_allclose(d, 1.09, atol=1e-12)
        u = (h[m] - c[m]) / 1.09
        g = u @ u.T
        np.testing.assert_allclose(g[np.triu_indices(4, 1)], -1.0 / 3.0, atol=1e-12)
    sites = np.array([[i, j, k] for i in range(4) for j in range(4) for k in range(3)], dtype=float) * 4.0
    assert np.abs(c - sites).max() <= 0.2
    mol_of = np.arange(48).tolist() + np.repeat(np.arange(48), 4).tolist()
    d = np.linalg.norm(xyz[:, None, :] - xyz[None, :, :], axis=2)
    other = np.array(mol_of)[:, None] != np.array(mol_of)[None, :]
    assert d[other].min() > 1.2
    syms2, xyz2 = molecules.methane_cluster_coords()
    np.testing.assert_array_equal(xyz, xyz2)
