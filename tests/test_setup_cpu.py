"""Host-side set-up checks (CPU): the native H2 construction reproduces the
reference's tree and pair lists, the struct layout matches the reference ABI,
and the representation survives save/load."""
import ctypes
import os

import numpy as np
import pytest

import h2eri_gb300 as hg
from conftest import GOLDEN, ref_lib_or_skip


def test_struct_layout_size():
    # struct H2ERI of the reference is 928 bytes on LP64 (src/H2ERI_typedef.h:14-131)
    assert ctypes.sizeof(hg.H2ERIStruct) == 928


def test_struct_layout_matches_reference():
    ref = ref_lib_or_skip()
    assert ref.oref_struct_size() == ctypes.sizeof(hg.H2ERIStruct)


def test_alk32_tree_counts(alk32):
    s = alk32.s
    # values printed by the reference's H2ERI_print_statistic for the same input
    assert (s.natom, s.nshell, s.num_bf) == (32, 126, 260)
    assert s.num_sp == 5968
    assert s.krnl_mat_size == 24498 == s.num_sp_bfp
    assert (s.n_node, s.max_level, s.min_adm_level) == (95, 4, 2)
    assert (s.n_r_adm_pair, s.n_r_inadm_pair, s.n_leaf_node) == (856, 447, 69)
    assert s.n_B == 856 and s.n_D == 69 + 447


def test_alk32_tree_equals_reference(alk32):
    """Same tree, pair lists and vector ranges as the reference's set-up run on
    the same molecule (reference sources compiled here with the integral shim)."""
    ref = ref_lib_or_skip()
    rh = ref.oref_build(os.path.join(GOLDEN, "alk32_ccpvdz.mol").encode(), 1e-10, 1e-10, 1e-6, 0)
    r = ctypes.cast(rh, ctypes.POINTER(hg.H2ERIStruct)).contents
    m = alk32.s
    for f in ("num_sp", "krnl_mat_size", "n_node", "n_leaf_node", "max_level", "min_adm_level",
              "n_r_adm_pair", "n_r_inadm_pair", "num_bf"):
        assert getattr(r, f) == getattr(m, f), f

    def arr(st, name, n):
        return np.ctypeslib.as_array(getattr(st, name), shape=(n,)).copy()

    nn = m.n_node
    for name, n in (("parent", nn), ("n_child", nn), ("node_level", nn), ("pt_cluster", 2 * nn),
                    ("mat_cluster", 2 * nn), ("r_adm_pairs", 2 * m.n_r_adm_pair),
                    ("r_inadm_pairs", 2 * m.n_r_inadm_pair), ("sp_bfp_sidx", m.num_sp + 1),
                    ("sp_shell_idx", 2 * m.num_sp), ("shell_bf_sidx", m.nshell + 1)):
        np.testing.assert_array_equal(arr(r, name, n), arr(m, name, n), err_msg=name)
    # ranks agree within a few (random sketches differ between the two builds)
    rU = ctypes.cast(r.U, ctypes.POINTER(ctypes.POINTER(hg.DenseMat)))
    mU = ctypes.cast(m.U, ctypes.POINTER(ctypes.POINTER(hg.DenseMat)))
    rr = np.array([rU[i].contents.ncol for i in range(nn)])
    mr = np.array([mU[i].contents.ncol for i in range(nn)])
    assert np.abs(rr - mr).max() <= 8
    assert abs(rr.sum() - mr.sum()) <= 0.02 * rr.sum()


def test_reference_coulomb_on_native_representation(alk32):
    """The reference's own H2ERI_build_Coulomb, run on the struct built by the
    native set-up, reproduces the reference's golden J (tests/test_J_input_mat.c)."""
    ref = ref_lib_or_skip()
    n = alk32.num_bf
    D = np.fromfile(os.path.join(GOLDEN, "D_alk32_ccpvdz.bin")).reshape(n, n)
    Jg = np.fromfile(os.path.join(GOLDEN, "J_alk32_ccpvdz.bin")).reshape(n, n)
    J = np.zeros_like(D)
    ref.H2ERI_build_Coulomb(alk32.handle, D.ctypes.data, J.ctypes.data)
    assert np.linalg.norm(J - Jg) / np.linalg.norm(Jg) < 2e-7


def test_save_load_roundtrip(alk26, tmp_path):
    p = str(tmp_path / "alk26.h2r")
    alk26.save(p)
    h2 = hg.H2ERI.load(p)
    try:
        for f in ("num_bf", "krnl_mat_size", "n_node", "n_B", "n_D", "n_leaf_node", "min_adm_level"):
            assert getattr(h2.s, f) == getattr(alk26.s, f)
        for kind in ("U", "B", "D"):
            a, b = alk26.blocks(kind), h2.blocks(kind)
            assert len(a) == len(b)
            for x, y in zip(a, b):
                assert x[:3] == y[:3]
                np.testing.assert_array_equal(x[3], y[3])
        np.testing.assert_array_equal(h2.int_array("plist", alk26.s.plist_sidx[alk26.s.nshell]),
                                      alk26.int_array("plist", alk26.s.plist_sidx[alk26.s.nshell]))
        assert list(h2.s.mat_size) == list(alk26.s.mat_size)
    finally:
        h2.destroy()


def test_load_rejects_bad_file(library, tmp_path):
    p = tmp_path / "bad.h2r"
    p.write_bytes(b"not a representation")
    with pytest.raises(hg.H2ERIError):
        hg.H2ERI.load(str(p))


def _blobs(raw):
    """(name, offset of element size, offset of data, element size, count) of
    every blob of a representation file (8-byte magic, then blobs of a 32-byte
    name, a 4-byte element size, an 8-byte count and the data)."""
    import struct
    out, pos = [], 8
    while pos + 44 <= len(raw):
        name = raw[pos:pos + 32].split(b"\0")[0].decode()
        es, cnt = struct.unpack_from("<IQ", raw, pos + 32)
        out.append((name, pos + 32, pos + 44, es, cnt))
        pos += 44 + es * cnt
    return out


def test_load_rejects_damaged_representation(small_mols, tmp_path):
    """Truncation, a block header that disagrees with its data, an inflated
    node count and a blob size beyond the file are all rejected with an error
    (nothing is read out of bounds); the undamaged file loads."""
    import struct
    good = tmp_path / "good.h2r"
    small_mols["C4H10"].save(str(good))
    raw = good.read_bytes()
    blobs = {b[0]: b for b in _blobs(raw)}

    def rejected(data, name):
        p = tmp_path / f"{name}.h2r"
        p.write_bytes(bytes(data))
        with pytest.raises(hg.H2ERIError):
            hg.H2ERI.load(str(p))

    rejected(raw[:len(raw) - 1000], "truncated")
    d = bytearray(raw)                       # first U block claims more elements than it has
    _, _, off, _, _ = blobs["U_hdr"]
    struct.pack_into("<i", d, off + 12, struct.unpack_from("<i", d, off + 12)[0] + 7)
    rejected(d, "header")
    d = bytearray(raw)                       # n_node far above the arrays' sizes
    _, _, off, _, _ = blobs["scalars"]
    struct.pack_into("<i", d, off + 9 * 4, 10 ** 6)
    rejected(d, "scalars")
    d = bytearray(raw)                       # a blob count beyond the end of the file
    _, cpos, _, _, _ = blobs["mat_cluster"]
    struct.pack_into("<Q", d, cpos + 4, 1 << 40)
    rejected(d, "count")
    h = hg.H2ERI.load(str(good))
    try:
        assert h.num_bf == small_mols["C4H10"].num_bf
    finally:
        h.destroy()


def test_block_storage_formats(alk32):
    """Blocks are dense (ld >= ncol) or low-rank (ld = -rank, U then V^T), and
    the low-rank form is only kept when it saves at least 20% (src/H2ERI_build_H2.c:869)."""
    n_lr = 0
    for kind in ("B", "D"):
        for nr, nc, ld, data in alk32.blocks(kind):
            if ld < 0:
                r = -ld
                n_lr += 1
                assert (nr + nc) * r <= nr * nc * 4 // 5
                assert data.size == (nr + nc) * r
            else:
                assert ld == nc and data.size == nr * nc
    assert n_lr > 0
