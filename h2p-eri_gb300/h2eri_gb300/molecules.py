"""Synthetic molecules in the reference's .mol format (H2P-ERI src/CMS.c:14-123).

Format: first line natom; per atom a header "<sym> <nshell> <nprimall> <nallprimg>",
a line "x y z" in Bohr, then nshell shell blocks "<type> <nprim> <ngen>" followed
by nprim lines "alpha c_1 .. c_ngen".

Basis data: cc-pVDZ blocks for C and H are taken verbatim from the reference
test molecule alk32_ccpvdz.mol (tests/golden). No other element is available.

Alkanes: straight-chain C_nH_{2n+2}, idealised all-trans zigzag with
C-C 1.54 A, C-H 1.09 A and tetrahedral angles, placed in the xz plane.
"""
import math
import os

import numpy as np

ANGSTROM_TO_BOHR = 1.8897261254578281
_GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                       "tests", "golden", "alk32_ccpvdz.mol")
_TETRA = math.acos(-1.0 / 3.0)   # 109.47 degrees


def _read_basis_blocks(path=_GOLDEN):
    """Return {symbol: (header_line, [shell lines])} for each element in a .mol file."""
    with open(path) as f:
        tok_lines = [ln.rstrip("\n") for ln in f]
    natom = int(tok_lines[0].split()[0])
    blocks = {}
    i = 1
    for _ in range(natom):
        header = tok_lines[i].split()
        sym, nshell = header[0], int(header[1])
        i += 2
        shell_lines = []
        for _s in range(nshell):
            sh = tok_lines[i].split()
            nprim = int(sh[1])
            shell_lines.extend(tok_lines[i:i + 1 + nprim])
            i += 1 + nprim
        if sym not in blocks:
            blocks[sym] = (" ".join(header), shell_lines)
    return blocks


def alkane_coords(n_carbon, cc=1.54, ch=1.09):
    """Cartesian coordinates (Angstrom) of an all-trans zigzag C_nH_{2n+2}.

    Returns (symbols, coords[natom, 3]); carbons first, then hydrogens.
    """
    if n_carbon < 1:
        raise ValueError("n_carbon must be >= 1")
    half = _TETRA / 2.0
    dx, dz = cc * math.sin(half), cc * math.cos(half)
    c_pos = [np.array([i * dx, 0.0, (i % 2) * dz]) for i in range(-1, n_carbon + 1)]
    carbons = c_pos[1:-1]
    yhat = np.array([0.0, 1.0, 0.0])
    hyd = []
    for i in range(n_carbon):
        c = c_pos[i + 1]
        left, right = c_pos[i], c_pos[i + 2]
        u1 = (left - c) / np.linalg.norm(left - c)
        u2 = (right - c) / np.linalg.norm(right - c)
        b = -(u1 + u2)
        b /= np.linalg.norm(b)
        for s in (+1.0, -1.0):
            hyd.append(c + ch * (math.cos(half) * b + s * math.sin(half) * yhat))
        if i == 0:
            hyd.append(c + ch * u1)          # terminal H along the virtual C-C bond
        if i == n_carbon - 1:
            hyd.append(c + ch * u2)
    syms = ["C"] * n_carbon + ["H"] * len(hyd)
    coords = np.array(carbons + hyd)
    return syms, coords


def write_mol(path, symbols, coords_angstrom):
    """Write a .mol file with cc-pVDZ (C, H) shells; coordinates given in Angstrom."""
    blocks = _read_basis_blocks()
    coords = np.asarray(coords_angstrom, dtype=np.float64) * ANGSTROM_TO_BOHR
    out = [str(len(symbols))]
    for s, xyz in zip(symbols, coords):
        if s not in blocks:
            raise ValueError(f"no basis data for element {s}")
        header, lines = blocks[s]
        out.append(header)
        out.append(f"{xyz[0]:.15f} {xyz[1]:.15f} {xyz[2]:.15f}")
        out.extend(lines)
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path


def write_alkane(path, n_carbon):
    syms, xyz = alkane_coords(n_carbon)
    return write_mol(path, syms, xyz)


def seeded_density(nbf, n_occ, seed):
    """D = C C^T with C an nbf x n_occ standard-normal matrix (numpy default_rng(seed))
    orthonormalised by a reduced QR. Symmetric float64, row-major."""
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((nbf, n_occ))
    q, _ = np.linalg.qr(c)
    return np.ascontiguousarray(q @ q.T)


def _random_rotation(rng):
    """A uniformly random rotation matrix (normalised Gaussian quaternion)."""
    q = rng.standard_normal(4)
    a, b, c, d = q / np.linalg.norm(q)
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def methane_cluster_coords(shape=(4, 4, 3), spacing=4.0, jitter=0.2, seed=5000, ch=1.09):
    """A 3-D cluster of CH4 molecules (Angstrom): one molecule per site of a
    cubic lattice of `shape` with `spacing` (4.0 A: liquid methane, 0.42
    g/cm^3, 63.4 A^3 per molecule), each centre moved by a uniform jitter in
    [-jitter, jitter] per axis and each molecule turned by a random rotation
    (numpy default_rng(seed)); tetrahedral CH4 with C-H = ch. It stands in for
    a water cluster where no oxygen basis data is available: the same 3-D
    neighbourhood structure (every molecule surrounded on all sides) with the
    C and H cc-pVDZ shells. 48 molecules give 1680 Cartesian basis functions.
    Returns (symbols, coords[natom, 3]), carbons first."""
    rng = np.random.default_rng(seed)
    tet = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64) / math.sqrt(3.0) * ch
    cs, hs = [], []
    for i in range(shape[0]):
        for j in range(shape[1]):
            for k in range(shape[2]):
                c = np.array([i, j, k], dtype=np.float64) * spacing + rng.uniform(-jitter, jitter, 3)
                R = _random_rotation(rng)
                cs.append(c)
                hs.extend(c + R @ t for t in tet)
    return ["C"] * len(cs) + ["H"] * len(hs), np.array(cs + hs)


def write_methane_cluster(path, shape=(4, 4, 3), spacing=4.0, jitter=0.2, seed=5000):
    syms, xyz = methane_cluster_coords(shape, spacing, jitter, seed)
    return write_mol(path, syms, xyz)
