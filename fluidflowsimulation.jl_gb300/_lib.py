"""ctypes binding of libffs.so (the C ABI declared in include/ffs.h)."""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int32, c_int64, c_void_p
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libffs.so"

FFS_OK = 0
ERRORS = {-1: "FFS_EINVAL", -2: "FFS_ENOMEM", -3: "FFS_ECUDA", -4: "FFS_ENAN", -5: "FFS_ETIMEDOUT",
          -6: "FFS_EUNSUPPORTED", -7: "FFS_ESTATE", -8: "FFS_ECANCELED"}
FFS_ETD3, FFS_AB3, FFS_EULER = 0, 1, 2
LES_MODELS = {"Smagorinsky": 0, "Vreman": 1, "productionViscosity": 2, "Silvis": 3, "stableNonLinear": 4,
              "dynamicSmagorinsky": 5, "piomelliSmagorinsky": 6}
FFS_FP64, FFS_FP32 = 0, 1

# Every symbol include/ffs.h declares (checked by the CPU test suite).
EXPORTS = [
    "ffs_params_default", "ffs_create", "ffs_set_fields", "ffs_initialize", "ffs_step", "ffs_finalize",
    "ffs_forcing_shells", "ffs_forcing_array", "ffs_capture_output", "ffs_output_field",
    "ffs_get_fields",
    "ffs_get_spectral", "ffs_set_spectral", "ffs_stats_header", "ffs_stats_ncols", "ffs_record_ncols",
    "ffs_stats_records", "ffs_stats", "ffs_spectrum", "ffs_spectrum_lengths", "ffs_spectrum_fields", "ffs_spectrum_records", "ffs_iteration", "ffs_time", "ffs_dt",
    "ffs_time_steps", "ffs_profile_kernels", "ffs_launches_per_step", "ffs_device_bytes", "ffs_tuning_report",
    "ffs_stream",
    "ffs_fourier_noalloc", "ffs_measure_fp64_peak", "ffs_last_error", "ffs_destroy",
    "ffs_server_default", "ffs_server_create", "ffs_submit", "ffs_poll", "ffs_wait", "ffs_fetch_stats",
    "ffs_fetch_fields", "ffs_release", "ffs_cancel", "ffs_server_pause", "ffs_server_stats", "ffs_server_tuning", "ffs_server_last_error", "ffs_server_destroy",
]
FFS_QUEUED, FFS_RUNNING = 1, 2


class FFSParams(ctypes.Structure):
    """Mirror of ``ffs_params`` (include/ffs.h)."""

    _fields_ = [
        ("nx", c_int32), ("ny", c_int32), ("nz", c_int32),
        ("lx", c_double), ("ly", c_double), ("lz", c_double),
        ("nu", c_double), ("cutoff", c_double),
        ("integrator", c_int32), ("variable_dt", c_int32),
        ("cfl", c_double), ("dt", c_double),
        ("hyperviscosity", c_int32), ("hv_nu", c_double), ("hv_m", c_int32),
        ("les", c_int32), ("smag_c", c_double), ("filter_width", c_double),
        ("density", c_int32), ("density_pr", c_double), ("density_gradient", c_double), ("gravity", c_double),
        ("gravity_dir", c_int32),
        ("forcing", c_int32), ("forcing_power", c_double), ("forcing_kf", c_double),
        ("precision", c_int32), ("dt_stat", c_int32), ("dt_spec", c_int32), ("write_time", c_int32),
        ("start", c_int64), ("start_time", c_double),
        ("device", c_int32), ("reference_cfl_slot", c_int32),
        ("stats_capacity", c_int32), ("spec_capacity", c_int32), ("kernel_variant", c_int32), ("autotune", c_int32),
        ("les_model", c_int32), ("les_cp", c_double), ("sandp_cb", c_double),
        ("passive_scalar", c_int32), ("scalar_pr", c_double), ("scalar_gradient", c_double), ("scalar_dir", c_int32),
        ("plane_forcing", c_int32), ("pf_tf", c_double), ("pf_alpha", c_double), ("pf_kf", c_double),
        ("pf_zf_tanh", c_int32), ("pf_qp", c_double), ("pf_qc", c_double), ("pf_qkf", c_double),
        ("les_test_width", c_double), ("les_cmin", c_double), ("spec_fil", c_double), ("les_dynp", c_int32),
        ("hv_kind", c_int32), ("hv_initk", c_double), ("hv_endk", c_double), ("rho_hv", c_int32), ("rho_hv_nu", c_double),
        ("rho_hv_m", c_int32), ("rho_hv_initk", c_double), ("rho_hv_endk", c_double),
        ("rho_les", c_int32), ("rho_les_c", c_double), ("radix_split", c_int32),
    ]


class FFSServerCfg(ctypes.Structure):
    """Mirror of ``ffs_server_cfg``."""
    _fields_ = [("device", c_int32), ("memory_budget", c_int64), ("max_active", c_int32), ("max_n", c_int32),
                ("autotune", c_int32), ("class_forms", c_int32)]


class FFSRequest(ctypes.Structure):
    """Mirror of ``ffs_request``."""
    _fields_ = [("params", FFSParams), ("u1", POINTER(c_double)), ("u2", POINTER(c_double)),
                ("u3", POINTER(c_double)), ("nt", c_int64), ("keep_fields", c_int32)]


class FFSResult(ctypes.Structure):
    """Mirror of ``ffs_result``."""
    _fields_ = [("status", c_int32), ("iteration", c_int64), ("time", c_double), ("dt", c_double),
                ("stats_rows", c_int64), ("record_ncols", c_int32), ("submit_s", c_double), ("admit_s", c_double),
                ("done_s", c_double)]


class FFSServerInfo(ctypes.Structure):
    """Mirror of ``ffs_server_info``."""
    _fields_ = [("batch_steps", c_int64), ("sim_steps", c_int64), ("active", c_int32), ("queued", c_int32),
                ("bytes_in_use", c_int64), ("peak_bytes", c_int64), ("peak_active", c_int32)]


_lib = None


def lib_available() -> bool:
    return LIB_PATH.exists()


def load() -> ctypes.CDLL:
    """Load libffs.so; raise loudly if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA engine first (python {HERE / 'build.py'})")
    L = ctypes.CDLL(str(LIB_PATH), mode=os.RTLD_LOCAL if hasattr(os, "RTLD_LOCAL") else 0)
    P = POINTER(FFSParams)
    H = c_void_p
    D = POINTER(c_double)
    sig = {
        "ffs_params_default": (c_int32, [P]),
        "ffs_create": (c_int32, [P, POINTER(c_void_p)]),
        "ffs_set_fields": (c_int32, [H, D, D, D, D, c_int32]),
        "ffs_initialize": (c_int32, [H]),
        "ffs_step": (c_int32, [H, c_int64]),
        "ffs_finalize": (c_int32, [H]),
        "ffs_forcing_shells": (c_int32, [H]),
        "ffs_forcing_array": (c_int32, [H, c_int32, D, c_int32, c_int32]),
        "ffs_capture_output": (c_int32, [H, c_int32]),
        "ffs_output_field": (c_int32, [H, c_int32, D, POINTER(c_int64)]),
        "ffs_get_fields": (c_int32, [H, D, D, D, D, c_int32]),
        "ffs_get_spectral": (c_int32, [H, c_int32, D]),
        "ffs_set_spectral": (c_int32, [H, c_int32, D]),
        "ffs_stats_header": (c_int32, [H, c_char_p, c_int64]),
        "ffs_stats_ncols": (c_int32, [H]),
        "ffs_record_ncols": (c_int32, [H]),
        "ffs_stats_records": (c_int64, [H, D, c_int64]),
        "ffs_stats": (c_int32, [H, D, c_int32]),
        "ffs_spectrum": (c_int32, [H, D, D, c_int64, c_int64]),
        "ffs_spectrum_lengths": (c_int32, [H, POINTER(c_int32), POINTER(c_int32)]),
        "ffs_spectrum_fields": (c_int32, [H, c_char_p, c_int64]),
        "ffs_spectrum_records": (c_int64, [H, D, c_int64]),
        "ffs_iteration": (c_int64, [H]),
        "ffs_time": (c_double, [H]),
        "ffs_dt": (c_double, [H]),
        "ffs_time_steps": (c_int32, [H, c_int64, D]),
        "ffs_profile_kernels": (c_int32, [H, c_int64, c_char_p, c_int64, D, c_int32, POINTER(c_int32)]),
        "ffs_launches_per_step": (c_int32, [H]),
        "ffs_device_bytes": (c_int64, [H]),
        "ffs_tuning_report": (c_int32, [H, c_char_p, c_int64]),
        "ffs_stream": (c_void_p, [H]),
        "ffs_fourier_noalloc": (c_int32, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_double, c_double,
                                         c_double, c_double, c_void_p]),
        "ffs_measure_fp64_peak": (c_int32, [c_int32, D, D]),
        "ffs_last_error": (c_char_p, [H]),
        "ffs_destroy": (None, [H]),
        "ffs_server_default": (c_int32, [POINTER(FFSServerCfg)]),
        "ffs_server_create": (c_int32, [POINTER(FFSServerCfg), POINTER(c_void_p)]),
        "ffs_submit": (c_int32, [H, POINTER(FFSRequest), POINTER(ctypes.c_uint64)]),
        "ffs_poll": (c_int32, [H, ctypes.c_uint64, POINTER(FFSResult)]),
        "ffs_wait": (c_int32, [H, ctypes.c_uint64, c_double, POINTER(FFSResult)]),
        "ffs_fetch_stats": (c_int64, [H, ctypes.c_uint64, D, c_int64]),
        "ffs_fetch_fields": (c_int32, [H, ctypes.c_uint64, D, D, D]),
        "ffs_release": (c_int32, [H, ctypes.c_uint64]),
        "ffs_cancel": (c_int32, [H, ctypes.c_uint64]),
        "ffs_server_pause": (c_int32, [H, c_int32]),
        "ffs_server_stats": (c_int32, [H, POINTER(FFSServerInfo)]),
        "ffs_server_tuning": (c_int64, [H, ctypes.c_char_p, c_int64]),
        "ffs_server_last_error": (c_char_p, [H]),
        "ffs_server_destroy": (None, [H]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class FFSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code
