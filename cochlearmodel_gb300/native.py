"""ctypes binding of libcochlea_gb300.so (the C ABI in include/cochlea_gb300.h).

The library is the only compute path: if it is missing or fails to load the
import of the solver raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

SECTIONS = 256
LAMBDA_COUNT = 3

UNIT_DTYPE = np.dtype([
    ("in_base", "<i8"), ("out_base", "<i8"), ("start", "<i4"), ("out_first", "<i4"),
    ("end", "<i4"), ("profile", "<i4"), ("mtt", "<f4"), ("mmspt", "<f4"),
])
STATS_DTYPE = np.dtype([
    ("substeps", "<i8"), ("iterations", "<i8"), ("sweeps", "<i8"),
    ("failed_samples", "<i4"), ("written_samples", "<i4"), ("status", "<i4"), ("pad_", "<i4"),
])
PROFILE_DTYPE = np.dtype([("dA", "<f8"), ("Wn", "<f8"), ("frequency", "<f8")])
assert UNIT_DTYPE.itemsize == 40 and STATS_DTYPE.itemsize == 40


class BMScalars(C.Structure):
    """cgb_bm_scalars: the float/int arguments of the BM step."""
    _fields_ = [(n, C.c_float) for n in (
        "w_ohc", "time_step", "time_step_out", "delta_x", "alpha_r", "Ts",
        "alpha_l", "alpha_s", "Gme", "a0", "a1", "a2", "sigma_ow", "eta_1", "eta_2",
        "dt_min", "dt_max")] + [(n, C.c_int32) for n in (
            "jacobi_fast", "jacobi_slow", "max_outer", "red_lanes", "jacobi_mode",
            "max_substeps_per_sample")] + [("jacobi_tol", C.c_float), ("jacobi_cap", C.c_int32),
                                           ("guess_mode", C.c_int32),
                                           ("learned_every", C.c_int32),
                                           ("controller", C.c_int32), ("arith", C.c_int32)]


class CGBError(RuntimeError):
    pass


_LIB = None

_p = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_d = C.c_double

_SIGS = {
    "cgb_last_error": (C.c_char_p, []),
    "cgb_abi_version": (_i, []),
    "cgb_kernel_launch_count": (_i64, []),
    "cgb_model_setup": (_i, [_p] * 11),
    "cgb_pack_sections": (_i, [_p] * 9),
    "cgb_block_partition": (_i, [_i, _i64, _i, _i, _p, _p, _p]),
    "cgb_check_units": (_i, [_p, _i, _i, _i64, _i64]),
    "cgb_bm_set_launch_shape": (_i, [_i]),
    "cgb_ihc_lambda_scratch_bytes": (_i64, [_i, _i, _i]),
    "cgb_ihc_lambda_upload_dev": (_i, [_p, _i, _p, _i, _p, _i, _p, _i64, _i64, _i, _p, _i64,
                                       _p]),
    "cgb_ihc_lambda_launch_dev": (_i, [_p, _i64, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p, _p, _i64,
                                       _p, _p, _i64, _p, _p]),
    "cgb_ihc_lambda_launch_mirror_dev": (_i, [_p, _i64, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p,
                                              _p, _i64, _p, _p, _i64, _p, _p, _i64, _p]),
    "cgb_ihc_set_fault_injection": (_i, [_i]),
    "cgb_ihc_set_run_length": (_i, [_i]),
    "cgb_ihc_lambda_noalloc_dev": (_i, [_p, _i64, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p, _p,
                                        _i64, _p, _p, _p]),
    "cgb_input_gen_dev": (_i, [_p, _i, _p, _p, _i, _i, _i, C.c_float, _d, _d, _d, _d, _p, _p]),
    "cgb_noise_normalization": (_i, [_p, _i, _d, _d, _i, _i, _i, _i, C.c_float, _p, _p]),
    "cgb_jnd_dev": (_i, [_p, _i64, _i, _i, _i, _i, _p, _p, _p, _p, _d, _d, _p, _p, _p, _p]),
    "cgb_jnd_final": (_i, [_p, _p, _i, _p, _d, _d, _p, _p]),
    "cgb_ihc_lambda_iir_scratch_bytes": (_i64, [_p, _i, _i, _i]),
    "cgb_ihc_lambda_iir_dev": (_i, [_p, _i64, _p, _i, _p, _p, _i, _p, _i, _p, _p, _i, _p, _p,
                                    _i64, _p, _p, _p, _i64, _p, _p]),
    "cgb_ihc_lambda_iir_stage_dev": (_i, [_p, _i64, _p, _i, _p, _p, _i, _p, _i, _p, _p, _i, _p,
                                          _p, _i64, _p, _p, _i, _p, _p, _i64, _p, _p]),
    "cgb_ihc_lambda_stage_dev": (_i, [_p, _i64, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p, _p,
                                      _i64, _p, _i, _p, _p, _i64, _p, _p]),
    "cgb_hearing_aid_dev": (_i, [_p, _i, _i, _p, _i, _p, _i, _p, _p]),
    "cgb_design_equiripple_lowpass": (_i, [_i, _d, _d, _d, _d, _p, _p, _p]),
    "cgb_complex_jnd": (_i, [_p, _i, _p, _p, _i, _i, _i, C.c_float, _p, _p, _p]),
    "cgb_jnd_batch_dev": (_i, [_p, _i64, _p, _i, _i, _p, _p, _d, _d, _p, _p, _p, _p]),
    "cgb_ihc_lambda_dev": (_i, [_p, _i64, _p, _i, _p, _i, _p, _i, _p, _p, _i, _p, _p, _i64, _p,
                                _p, _i64, _p, _p]),
    "cgb_bm_launch_shape_count": (_i, []),
    "cgb_bm_run_dev": (_i, [_p, _p, _i, C.POINTER(BMScalars), _p, _i, _p, _i64, _p, _i64,
                            _p, _p, _p, _p, _p]),
    "cgb_bm_run_ex_dev": (_i, [_p, _p, _i, C.POINTER(BMScalars), _p, _i, _p, _i64, _p, _i64,
                               _p, _p, _p, _p, C.c_void_p, _p]),
    "cgb_ws_blob_bytes": (_i, []),
    "cgb_ws_blobT_bytes": (_i, []),
    "cgb_ws_param_count": (_i, []),
    "cgb_ws_pack_dev": (_i, [_p, C.c_float, C.c_float, _p, _p, _p]),
    "cgb_ws_prepare_dev": (_i, [_p, _i, _p, C.c_float, _p, _p, _p, _p, _p]),
    "cgb_ws_forward_dev": (_i, [_p, _p, _i, _p, _p, _p]),
    "cgb_ws_loss_dev": (_i, [_p, _p, _i, C.c_float, _p, _p, _p]),
    "cgb_ws_backward_dev": (_i, [_p, _p, _p, _i, _p, _p]),
    "cgb_ws_wgrad_dev": (_i, [_p, _p, _p, _p, _i, _p, _i, _p, _p]),
    "cgb_ws_adam_dev": (_i, [_p, _p, _p, _p, _i, C.c_float, C.c_float, C.c_float, C.c_float,
                             _p]),
    "cgb_ws_infer_dev": (_i, [_p, _p, _i, _p, _p]),
}


JND_INTERVAL_DTYPE = np.dtype([("row", np.int64), ("ref_row", np.int64), ("dA", np.float64),
                               ("len", np.int32), ("out", np.int32)])
assert JND_INTERVAL_DTYPE.itemsize == 32


class BMExtras(C.Structure):
    """cgb_bm_extras: network weights, training-record logging and the host
    mirror of the velocity output (fields left at zero are unused)."""
    _fields_ = [("d_ws_blob", C.c_void_p), ("d_log", C.c_void_p), ("log_cap", C.c_int64),
                ("log_every", C.c_int32), ("pad_", C.c_int32), ("d_log_count", C.c_void_p),
                ("h_out_bytes", C.c_int64), ("h_out", C.c_void_p)]


def lib_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads the native library (building it first when allowed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not path.exists() or not _build.up_to_date():
        if not build_if_missing or os.environ.get("CGB_NO_BUILD"):
            raise CGBError(f"native library missing or stale: {path}")
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = load().cgb_last_error().decode(errors="replace")
        raise CGBError(f"{what or 'cochlea_gb300'} failed ({status}): {msg}")


def check_host_mirror(t, like, name: str):
    """A host mirror receives a kernel's stores directly, so its size must be
    exactly that of the device buffer it mirrors: a pinned, contiguous CPU
    tensor of the same shape and dtype (torch's pin_memory() maps it into the
    device address space at the same address)."""
    ok = (t is not None and t.device.type == "cpu" and t.is_pinned() and t.is_contiguous()
          and t.dtype == like.dtype and tuple(t.shape) == tuple(like.shape))
    if not ok:
        raise ValueError(f"{name} must be a pinned contiguous CPU tensor of shape "
                         f"{tuple(like.shape)} and dtype {like.dtype}")
    return t


def ptr(a) -> int:
    """Address of a numpy array or a torch tensor's storage."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
