"""ctypes bindings of libsgdg (include/sgdg.h).  No fallback: if the library
cannot be built or loaded, or a compute call finds no GPU, an exception is
raised."""
import ctypes
import os

import numpy as np

from . import build as _build

OK, EINVAL, ENOMEM_BUDGET, ETIMEOUT, ECUDA, ECANCELLED, ENOGPU, EUNSUPPORTED, EIO, ENONFINITE = range(10)
SCHEMES = {"sparse": 0, "full": 1}
METHODS = {"plain": 0, "matfree": 1}
BASES = {"hier": 0, "pos": 1}
KIND_ADVECT, KIND_WAVE = 0, 1
OP_LAPLACIAN, OP_WAVE_RHS = 0, -1

# every symbol include/sgdg.h declares
EXPORTS = [
    "sgdg_version", "sgdg_last_error", "sgdg_get_size", "sgdg_index_map", "sgdg_dg_coeffs", "sgdg_dlf_1d_nnz",
    "sgdg_dlf_1d_export", "sgdg_op_create", "sgdg_op_create_1d", "sgdg_op_destroy", "sgdg_op_size", "sgdg_op_nnz",
    "sgdg_op_export_csr", "sgdg_op_device_nnz", "sgdg_op_export_device_csr", "sgdg_apply", "sgdg_apply_device", "sgdg_apply_noalloc", "sgdg_wave_evolve",
    "sgdg_advect_evolve", "sgdg_op_plain_steps_device", "sgdg_debug_bounds", "sgdg_vcoeffs_contract",
    "sgdg_batch_create", "sgdg_batch_destroy", "sgdg_batch_add", "sgdg_batch_remove", "sgdg_batch_set_stream",
    "sgdg_batch_step", "sgdg_batch_get_state", "sgdg_batch_state_size", "sgdg_batch_total_size",
    "sgdg_batch_upload", "sgdg_batch_download", "sgdg_batch_step_host", "sgdg_batch_step_info", "sgdg_batch_autotune",
    "sgdg_batch_add_vlasov",
    "sgdg_tile_shape", "sgdg_set_tile_shape", "sgdg_clear_tile_shapes", "sgdg_server_snapshot",
    "sgdg_transform_1d_nnz", "sgdg_transform_1d_export", "sgdg_transform_nnz", "sgdg_transform_export",
    "sgdg_transform_device_export",
    "sgdg_vlasov_create", "sgdg_vlasov_destroy", "sgdg_vlasov_size", "sgdg_vlasov_v_point",
    "sgdg_vlasov_transform_nnz", "sgdg_vlasov_transform_export", "sgdg_vlasov_rhs", "sgdg_vlasov_evolve",
    "sgdg_vlasov_write_h5",
    "sgdg_server_create", "sgdg_server_destroy", "sgdg_server_set_stream", "sgdg_server_clock",
    "sgdg_server_submit", "sgdg_server_tick", "sgdg_server_status", "sgdg_server_result", "sgdg_server_cancel",
    "sgdg_server_counts",
    "sgdg_evaluate", "sgdg_evaluate_device", "sgdg_tensor_sum", "sgdg_selftest_bounded_wait", "sgdg_selftest_convert", "sgdg_worklist_dryrun", "sgdg_set_hbm_budget", "sgdg_hbm_in_use", "sgdg_sync",
]
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = range(5)


class SGDGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("sgdg error %d: %s" % (code, msg))
        self.code = code


_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_ci = ctypes.c_int
_c64 = ctypes.c_int64
_cd = ctypes.c_double

_lib = None


def _sig(L, name, args):
    f = getattr(L, name)
    f.argtypes = args
    f.restype = ctypes.c_int


def lib(build=True):
    """Load (building first if needed) the in-tree libsgdg.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise OSError("libsgdg.so not built: %s" % path)
    L = ctypes.CDLL(path)
    _sig(L, "sgdg_version", [ctypes.c_char_p, ctypes.c_size_t])
    _sig(L, "sgdg_last_error", [ctypes.c_char_p, ctypes.c_size_t])
    _sig(L, "sgdg_get_size", [_ci, _ci, _ci, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_index_map", [_ci, _ci, _ci, _ci, _i32p, _i32p, _i32p])
    _sig(L, "sgdg_dg_coeffs", [_ci, _f64p])
    _sig(L, "sgdg_dlf_1d_nnz", [_ci, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_dlf_1d_export", [_ci, _ci, _i64p, _i32p, _f64p])
    _sig(L, "sgdg_op_create", [_ci, _ci, _ci, _ci, ctypes.POINTER(_vp)])
    _sig(L, "sgdg_op_create_1d", [_ci, _ci, _ci, ctypes.POINTER(_vp)])
    _sig(L, "sgdg_op_destroy", [_vp])
    _sig(L, "sgdg_op_size", [_vp, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_op_nnz", [_vp, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_op_export_csr", [_vp, _ci, _i64p, _i32p, _f64p])
    _sig(L, "sgdg_op_device_nnz", [_vp, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_op_export_device_csr", [_vp, _ci, _i64p, _i32p, _f64p])
    _sig(L, "sgdg_apply", [_vp, _ci, _ci, _f64p, _f64p])
    _sig(L, "sgdg_apply_device", [_vp, _ci, _ci, _vp, _vp, _vp])
    _sig(L, "sgdg_apply_noalloc", [_ci, _ci, _ci, _ci, _ci, _vp, _vp, _vp])
    _sig(L, "sgdg_wave_evolve", [_vp, _f64p, _f64p, _cd, _cd, _c64, _ci, _ci, _f64p, _f64p])
    _sig(L, "sgdg_advect_evolve", [_vp, _f64p, _f64p, _cd, _cd, _c64, _ci, _ci, _f64p, _f64p])
    _sig(L, "sgdg_op_plain_steps_device", [_vp, _ci, _c64, _vp, _cd, _c64, _vp])
    _sig(L, "sgdg_debug_bounds", [ctypes.POINTER(_ci), ctypes.POINTER(_c64), _ci])
    _sig(L, "sgdg_vcoeffs_contract", [_ci, _ci, _ci, _ci, _i32p, _f64p, _f64p, _f64p])
    _sig(L, "sgdg_transform_1d_nnz", [_ci, _ci, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_transform_1d_export", [_ci, _ci, _ci, _i64p, _i32p, _f64p])
    _sig(L, "sgdg_transform_nnz", [_ci, _ci, _ci, _ci, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_transform_export", [_ci, _ci, _ci, _ci, _ci, _i64p, _i32p, _f64p])
    _sig(L, "sgdg_transform_device_export", [_ci, _ci, _ci, _ci, _ci, ctypes.POINTER(_c64), _vp, _vp, _vp])
    _sig(L, "sgdg_vlasov_create", [_ci, _ci, _ci, _ci, ctypes.POINTER(_vp)])
    _sig(L, "sgdg_vlasov_destroy", [_vp])
    _sig(L, "sgdg_vlasov_size", [_vp, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_vlasov_v_point", [_vp, _f64p])
    _sig(L, "sgdg_vlasov_transform_nnz", [_vp, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_vlasov_transform_export", [_vp, _ci, _i64p, _i32p, _f64p])
    _sig(L, "sgdg_vlasov_rhs", [_vp, _f64p, _f64p, _f64p])
    _sig(L, "sgdg_vlasov_evolve", [_vp, _f64p, _f64p, _cd, _cd, _c64, _ci, _ci, _f64p, _f64p])
    _sig(L, "sgdg_vlasov_write_h5", [_vp, ctypes.c_char_p, _c64, _vp, _vp])
    _sig(L, "sgdg_batch_add_vlasov", [_vp, _ci, _ci, _ci, _ci, _cd, _f64p, _f64p, ctypes.POINTER(_ci)])
    _sig(L, "sgdg_evaluate", [_ci, _ci, _ci, _ci, _f64p, _c64, _f64p, _f64p])
    _sig(L, "sgdg_evaluate_device", [_ci, _ci, _ci, _ci, _vp, _c64, _vp, _vp, _vp])
    _sig(L, "sgdg_tensor_sum", [_ci, _ci, _ci, _ci, _ci, _f64p, _f64p, _f64p])
    _sig(L, "sgdg_selftest_bounded_wait", [ctypes.POINTER(_cd)])
    _sig(L, "sgdg_selftest_convert", [_f64p, _c64, ctypes.POINTER(_c64), ctypes.POINTER(_c64)])
    _sig(L, "sgdg_worklist_dryrun", [_ci, _vp, _ci, _ci, _ci, _vp, _c64, ctypes.POINTER(_c64), ctypes.POINTER(_ci), _vp, _vp, _c64, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_server_create", [_ci, ctypes.POINTER(_vp)])
    _sig(L, "sgdg_server_destroy", [_vp])
    _sig(L, "sgdg_server_set_stream", [_vp, _vp])
    _sig(L, "sgdg_server_clock", [_vp, ctypes.POINTER(_cd)])
    _sig(L, "sgdg_server_submit", [_vp, _ci, _ci, _ci, _ci, _ci, _vp, _cd, _f64p, _c64, _cd, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_server_tick", [_vp, ctypes.POINTER(_ci)])
    _sig(L, "sgdg_server_status", [_vp, _c64, ctypes.POINTER(_ci), ctypes.POINTER(_c64), ctypes.POINTER(_cd),
                                   ctypes.POINTER(_cd), ctypes.POINTER(_cd)])
    _sig(L, "sgdg_server_result", [_vp, _c64, _f64p])
    _sig(L, "sgdg_server_cancel", [_vp, _c64])
    _sig(L, "sgdg_server_snapshot", [_vp, _c64, _f64p, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_server_counts", [_vp, ctypes.POINTER(_c64), ctypes.POINTER(_c64), ctypes.POINTER(_c64),
                                   ctypes.POINTER(_cd)])
    _sig(L, "sgdg_batch_autotune", [_vp, ctypes.POINTER(_ci)])
    _sig(L, "sgdg_tile_shape", [_ci, _ci, ctypes.POINTER(_ci), ctypes.POINTER(_ci), ctypes.POINTER(_ci)])
    _sig(L, "sgdg_set_tile_shape", [_ci, _ci, _ci, _ci])
    _sig(L, "sgdg_clear_tile_shapes", [])
    _sig(L, "sgdg_batch_create", [ctypes.POINTER(_vp)])
    _sig(L, "sgdg_batch_destroy", [_vp])
    _sig(L, "sgdg_batch_add", [_vp, _ci, _ci, _ci, _ci, _ci, _vp, _cd, _f64p, ctypes.POINTER(_ci)])
    _sig(L, "sgdg_batch_remove", [_vp, _ci])
    _sig(L, "sgdg_batch_set_stream", [_vp, _vp])
    _sig(L, "sgdg_batch_step", [_vp, _c64])
    _sig(L, "sgdg_batch_get_state", [_vp, _ci, _f64p])
    _sig(L, "sgdg_batch_state_size", [_vp, _ci, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_batch_total_size", [_vp, ctypes.POINTER(_c64)])
    _sig(L, "sgdg_batch_upload", [_vp, _vp])
    _sig(L, "sgdg_batch_download", [_vp, _vp])
    _sig(L, "sgdg_batch_step_host", [_vp, _vp, _vp, _c64, _ci])
    _sig(L, "sgdg_batch_step_info", [_vp, ctypes.POINTER(_c64), ctypes.POINTER(_cd)])
    _sig(L, "sgdg_set_hbm_budget", [_c64])
    _sig(L, "sgdg_hbm_in_use", [ctypes.POINTER(_c64)])
    _sig(L, "sgdg_sync", [])
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().sgdg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code):
    if code != OK:
        raise SGDGError(code, last_error())
