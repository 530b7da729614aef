"""Python host side of h2eri_gb300: ctypes bindings over the C ABI in
include/h2eri_gb300.h (libh2eri_gb300.so), mirroring the reference call
sequence (H2P-ERI tests/test_J_input_mat.c:17-50):

    h = H2ERI(qr_tol=1e-6)            # H2ERI_init
    h.read_mol("x.mol")               # CMS_read_mol_file
    h.process_shells(); h.partition(); h.build_h2()
    J = h.build_coulomb(D)            # H2ERI_build_Coulomb (GPU)
    K = h.build_exchange(D)           # H2ERI_build_exchange (GPU)

The hot path only exists on the GPU; there is no CPU fallback in this
package. Calls raise H2ERIError with the library's message on failure.
"""
import ctypes
import os

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "lib", "libh2eri_gb300.so")

FP64 = 0
MIXED = 1

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class H2ERIStruct(ctypes.Structure):
    """Mirror of struct H2ERI (include/h2eri_types.h; reference layout
    H2P-ERI src/H2ERI_typedef.h:14-131)."""
    _fields_ = (
        [(n, ctypes.c_int) for n in ("natom", "nshell", "max_am", "max_shell_nbf", "num_bf", "num_sp",
                                     "num_sp_bfp", "pp_npts_layer", "pp_nlayer_ext")]
        + [(n, _c_int_p) for n in ("shell_bf_sidx", "sp_nbfp", "sp_bfp_sidx", "sp_shell_idx", "index_seq",
                                   "node_adm_pairs", "node_adm_pairs_sidx", "node_inadm_pairs",
                                   "node_inadm_pairs_sidx", "plist", "plist_idx", "plist_sidx", "dlist",
                                   "dlist_sidx")]
        + [("thread_Kmat_workbuf", _vp), ("scr_tol", ctypes.c_double), ("ext_tol", ctypes.c_double)]
        + [(n, _c_dbl_p) for n in ("sp_center", "sp_extent", "box_extent", "unc_denmat_x", "H2_matvec_y")]
        + [(n, _vp) for n in ("shells", "sp_shells", "sp", "J_pair", "J_row", "ovlp_ff_idx", "simint_buffs",
                              "eri_batch_buffs", "c_B_blks", "c_D_blks", "thread_buffs")]
        + [(n, ctypes.c_int) for n in ("n_thread", "pt_dim", "xpt_dim", "krnl_dim", "QR_stop_type",
                                       "QR_stop_rank", "n_point", "krnl_mat_size", "max_leaf_points", "n_node",
                                       "root_idx", "n_leaf_node", "max_child", "max_neighbor", "max_level",
                                       "min_adm_level", "n_r_inadm_pair", "n_r_adm_pair", "n_UJ", "n_B", "n_D",
                                       "BD_JIT", "print_timers", "print_dbginfo")]
        + [(n, _c_int_p) for n in ("parent", "children", "pt_cluster", "mat_cluster", "n_child", "node_level",
                                   "node_height", "level_n_node", "level_nodes", "height_n_node",
                                   "height_nodes", "r_inadm_pairs", "r_adm_pairs", "node_inadm_lists",
                                   "node_n_r_inadm", "node_n_r_adm", "coord_idx", "B_p2i_rowptr",
                                   "B_p2i_colidx", "B_p2i_val", "D_p2i_rowptr", "D_p2i_colidx", "D_p2i_val",
                                   "B_nrow", "B_ncol", "D_nrow", "D_ncol")]
        + [("B_ptr", _vp), ("D_ptr", _vp), ("max_leaf_size", ctypes.c_double), ("QR_stop_tol", ctypes.c_double)]
        + [(n, _c_dbl_p) for n in ("coord", "coord0", "enbox", "root_enbox", "B_data", "D_data")]
        + [(n, _vp) for n in ("B_blk", "D_blk0", "D_blk1", "U", "y0", "y1")]
        + [("n_matvec", ctypes.c_int), ("mat_size", ctypes.c_size_t * 11), ("timers", ctypes.c_double * 11)]
    )


class DenseMat(ctypes.Structure):
    _fields_ = [("nrow", ctypes.c_int), ("ncol", ctypes.c_int), ("ld", ctypes.c_int), ("size", ctypes.c_int),
                ("data", _c_dbl_p)]


# exported symbols of the C ABI: name -> (restype, argtypes)
SIGNATURES = {
    "H2ERI_init": (None, [ctypes.POINTER(_vp), ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "H2ERI_destroy": (None, [_vp]),
    "H2ERI_print_statistic": (None, [_vp]),
    "CMS_read_mol_file": (None, [ctypes.c_char_p, _c_int_p, _c_int_p, ctypes.POINTER(_vp)]),
    "CMS_destroy_shells": (None, [ctypes.c_int, _vp]),
    "H2ERI_process_shells": (None, [_vp]),
    "H2ERI_partition": (None, [_vp]),
    "H2ERI_build_H2": (None, [_vp, ctypes.c_int]),
    "H2ERI_matvec": (None, [_vp, _vp, _vp]),
    "H2ERI_build_Coulomb": (None, [_vp, _vp, _vp]),
    "H2ERI_build_exchange": (None, [_vp, _vp, _vp]),
    "H2ERI_exchange_workbuf_init": (None, [_vp]),
    "H2ERI_exchange_workbuf_free": (None, [_vp]),
    "H2E_reset_timers": (None, [_vp]),
    "H2ERI_gpu_upload": (ctypes.c_int, [_vp]),
    "H2ERI_gpu_release": (None, [_vp]),
    "H2ERI_gpu_set_precision": (ctypes.c_int, [_vp, ctypes.c_int]),
    "H2ERI_gpu_last_error": (ctypes.c_char_p, []),
    "H2ERI_gpu_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_longlong]),
    "H2ERI_matvec_multi": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    "H2ERI_matvec_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    "H2ERI_build_Coulomb_multi": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    "H2ERI_build_Coulomb_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    "H2ERI_build_Coulomb_batch": (ctypes.c_int, [ctypes.c_int, _vp, _vp, _vp, _vp, _vp]),
    "H2ERI_build_exchange_multi": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    "H2ERI_build_exchange_device": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "H2ERI_gpu_exchange_report": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "H2ERI_exchange_plan_check": (ctypes.c_int, [_vp, ctypes.c_double, _vp, ctypes.c_int]),
    "H2ERI_gpu_set_exchange_memory": (ctypes.c_int, [_vp, ctypes.c_double]),
    "H2ERI_gpu_report": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "H2ERI_matvec_device_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "H2ERI_gpu_check": (ctypes.c_int, [_vp]),
    "H2ERI_gpu_autotune": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int]),
    "H2ERI_gpu_selftest_wait_timeout_async": (ctypes.c_int, [_vp, ctypes.c_longlong, _vp]),
    "H2ERI_gpu_selftest_persist_timeout": (ctypes.c_int, [_vp, ctypes.c_longlong]),
    "H2ERI_gpu_setup_eri_check": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "H2ERI_gpu_setup_u_check": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "H2ERI_gpu_drop_fp64": (ctypes.c_int, [_vp]),
    "H2ERI_save_representation": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "H2ERI_load_representation": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
}

_LIB = None


class H2ERIError(RuntimeError):
    pass


def lib():
    """Load libh2eri_gb300.so (built in-tree by h2eri_gb300.build). Raises if absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise H2ERIError(f"{LIB_PATH} missing: run h2eri_gb300.build.build() first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _check(rc, what):
    if rc != 0:
        msg = lib().H2ERI_gpu_last_error().decode()
        raise H2ERIError(f"{what} failed ({rc}): {msg}")


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class H2ERI:
    """One H2 representation of the ERI tensor (wraps an H2ERI_p)."""

    def __init__(self, scr_tol=1e-10, ext_tol=1e-10, qr_tol=1e-6, _handle=None):
        L = lib()
        if _handle is None:
            h = _vp()
            L.H2ERI_init(ctypes.byref(h), scr_tol, ext_tol, qr_tol)
            self.handle = h
        else:
            self.handle = _handle
        self.s = ctypes.cast(self.handle, ctypes.POINTER(H2ERIStruct)).contents

    # ---- set-up (host, once per geometry) ----
    def read_mol(self, path):
        s = self.s
        natom, nshell, shells = ctypes.c_int(), ctypes.c_int(), _vp()
        lib().CMS_read_mol_file(os.fsencode(path), ctypes.byref(natom), ctypes.byref(nshell), ctypes.byref(shells))
        s.natom, s.nshell, s.shells = natom.value, nshell.value, shells
        return self

    def process_shells(self):
        lib().H2ERI_process_shells(self.handle)
        return self

    def partition(self):
        lib().H2ERI_partition(self.handle)
        return self

    def build_h2(self):
        lib().H2ERI_build_H2(self.handle, 0)
        return self

    @classmethod
    def from_mol(cls, path, qr_tol=1e-6, scr_tol=1e-10, ext_tol=1e-10):
        return cls(scr_tol, ext_tol, qr_tol).read_mol(path).process_shells().partition().build_h2()

    @classmethod
    def load(cls, path):
        h = _vp()
        _check(lib().H2ERI_load_representation(os.fsencode(path), ctypes.byref(h)), "load_representation")
        return cls(_handle=h)

    def save(self, path):
        _check(lib().H2ERI_save_representation(self.handle, os.fsencode(path)), "save_representation")

    # ---- properties ----
    @property
    def num_bf(self):
        return self.s.num_bf

    @property
    def krnl_mat_size(self):
        return self.s.krnl_mat_size

    @property
    def mat_size(self):
        return list(self.s.mat_size)

    def blocks(self, kind):
        """Host blocks as (nrow, ncol, ld, ndarray) tuples; kind in U, B, D."""
        s = self.s
        n, ptr = {"U": (s.n_UJ, s.U), "B": (s.n_B, s.c_B_blks), "D": (s.n_D, s.c_D_blks)}[kind]
        arr = ctypes.cast(ptr, ctypes.POINTER(ctypes.POINTER(DenseMat)))
        out = []
        for i in range(n):
            m = arr[i].contents
            cnt = (m.nrow + m.ncol) * (-m.ld) if m.ld < 0 else m.nrow * m.ncol
            data = np.ctypeslib.as_array(m.data, shape=(cnt,)).copy() if cnt > 0 else np.zeros(0)
            out.append((m.nrow, m.ncol, m.ld, data))
        return out

    def int_array(self, name, n):
        p = getattr(self.s, name)
        return np.ctypeslib.as_array(p, shape=(n,)).copy() if n > 0 else np.zeros(0, np.int32)

    # ---- hot path (GPU) ----
    def upload(self):
        _check(lib().H2ERI_gpu_upload(self.handle), "gpu_upload")

    def set_precision(self, mode):
        _check(lib().H2ERI_gpu_set_precision(self.handle, mode), "gpu_set_precision")

    def matvec(self, x):
        x = _f64(x)
        nvec = 1 if x.ndim == 1 else x.shape[0]
        y = np.empty_like(x)
        _check(lib().H2ERI_matvec_multi(self.handle, nvec, x.ctypes.data, y.ctypes.data), "matvec")
        return y

    def build_coulomb(self, D):
        D = _f64(D)
        n_den = 1 if D.ndim == 2 else D.shape[0]
        J = np.empty_like(D)
        _check(lib().H2ERI_build_Coulomb_multi(self.handle, n_den, D.ctypes.data, J.ctypes.data), "build_Coulomb")
        return J

    def build_exchange(self, D):
        D = _f64(D)
        n_den = 1 if D.ndim == 2 else D.shape[0]
        K = np.empty_like(D)
        _check(lib().H2ERI_build_exchange_multi(self.handle, n_den, D.ctypes.data, K.ctypes.data), "build_exchange")
        return K

    def exchange_report(self):
        """Exchange-plan figures (see H2ERI_gpu_exchange_report)."""
        out = np.zeros(8)
        n = lib().H2ERI_gpu_exchange_report(self.handle, out.ctypes.data, 8)
        if n < 0:
            _check(-n, "gpu_exchange_report")
        keys = ["flops", "ms_last", "n_ranges", "work_bytes", "near_items", "launches", "tensor_cores"]
        return dict(zip(keys, out[:n].tolist()))

    def report(self):
        """Device-copy figures (see H2ERI_gpu_report in include/h2eri_gb300.h)."""
        out = np.zeros(23)
        n = lib().H2ERI_gpu_report(self.handle, out.ctypes.data, 23)
        if n < 0:
            _check(-n, "gpu_report")
        keys = ["launches_per_matvec", "alg_matrix_bytes", "alg_vector_bytes", "alg_flops", "arena_U", "arena_B",
                "arena_D", "ms_fwd", "ms_mid", "ms_bwd", "ms_den", "ms_total", "precision", "noalloc_scratch_doubles",
                "tile_rows", "tiles_per_cta", "nf_concurrent", "mma_min_vec", "mma_grid_div", "persist",
                "px_items", "px_grid", "px_sim_ms"]
        return dict(zip(keys, out[:n].tolist()))

    def autotune(self, n_den=1):
        """Time every candidate launch configuration at n_den densities per
        launch and keep the fastest (H2ERI_gpu_autotune); returns a dict."""
        out = np.zeros(64)
        m = lib().H2ERI_gpu_autotune(self.handle, n_den, out.ctypes.data, 64)
        if m < 0:
            _check(-m, "gpu_autotune")
        return {"ms_best": out[0], "ms_before": out[1], "candidates": int(out[2]),
                "choice": {"tile_rows": int(out[3]), "tiles_per_cta": int(out[4]), "nf_concurrent": int(out[5]),
                           "mma_min_vec": int(out[6]), "mma_grid_div": int(out[7]), "persist": int(out[8])},
                "ms_candidates": out[9:m].tolist()}

    def print_statistic(self):
        lib().H2ERI_print_statistic(self.handle)

    def destroy(self):
        if self.handle:
            lib().H2ERI_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


from . import molecules  # noqa: E402,F401
