"""ctypes binding of libcpml.so (include/cpml.h).

Loads the in-tree library built by ``seismic_cpml_gb300.build``. There is no
fallback: if the library is missing the import of the solver fails loudly.
"""
from __future__ import annotations

import ctypes
import os

from .params import CpmlParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcpml.so")

OK = 0
KERNEL_AUTO, KERNEL_TWO_SWEEP, KERNEL_FUSED, KERNEL_PERSISTENT, KERNEL_CLUSTER = 0, 1, 2, 3, 4
ERR = {-1: "INVALID", -2: "CFL", -3: "OOM", -4: "UNSTABLE", -5: "TIMEOUT", -6: "CUDA",
       -7: "NOT_READY", -8: "IO", -9: "RANGE"}

# (name, restype, argtypes) for every entry point declared in include/cpml.h
_P = ctypes.POINTER
_dp, _fp, _ip, _vp = _P(ctypes.c_double), _P(ctypes.c_float), _P(ctypes.c_int), ctypes.c_void_p
_h = ctypes.c_void_p
SIGNATURES = [
    ("cpml_params_default_2d", ctypes.c_int, [_P(CpmlParams)]),
    ("cpml_params_default_3d", ctypes.c_int, [_P(CpmlParams)]),
    ("cpml_params_default_2d_fourth", ctypes.c_int, [_P(CpmlParams)]),
    ("cpml_params_default_2d_split", ctypes.c_int, [_P(CpmlParams)]),
    ("cpml_courant", ctypes.c_double, [_P(CpmlParams), ctypes.c_double]),
    ("cpml_nearest_gridpoint", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                              _ip, _ip]),
    ("cpml_pml_profile", ctypes.c_int, [_P(CpmlParams), ctypes.c_int, ctypes.c_int] + [_dp] * 10),
    ("cpml_create", ctypes.c_int, [_P(CpmlParams), _P(_h)]),
    ("cpml_set_model", ctypes.c_int, [_h, _fp, _fp, _fp]),
    ("cpml_set_receivers", ctypes.c_int, [_h, ctypes.c_int, _ip, _ip, _ip]),
    ("cpml_reset", ctypes.c_int, [_h]),
    ("cpml_run", ctypes.c_int, [_h, ctypes.c_int]),
    ("cpml_status", ctypes.c_int, [_h, _ip, _dp]),
    ("cpml_get_seismograms", ctypes.c_int, [_h, _dp, _dp, _dp]),
    ("cpml_get_energy", ctypes.c_int, [_h, _dp, _dp]),
    ("cpml_get_field", ctypes.c_int, [_h, ctypes.c_int, _fp]),
    ("cpml_get_plane", ctypes.c_int, [_h, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp]),
    ("cpml_set_field", ctypes.c_int, [_h, ctypes.c_int, _fp]),
    ("cpml_state_size", ctypes.c_int, [_h, _P(ctypes.c_size_t)]),
    ("cpml_save_state", ctypes.c_int, [_h, _vp, ctypes.c_size_t]),
    ("cpml_load_state", ctypes.c_int, [_h, _vp, ctypes.c_size_t]),
    ("cpml_algorithmic_bytes_per_step", ctypes.c_double, [_h]),
    ("cpml_last_run_ms", ctypes.c_int, [_h, _dp]),
    ("cpml_get_stream", ctypes.c_int, [_h, _P(ctypes.c_void_p)]),
    ("cpml_set_tuning", ctypes.c_int, [_h, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("cpml_get_tuning", ctypes.c_int, [_h, _ip, _ip, _ip, _ip]),
    ("cpml_launches_per_step", ctypes.c_int, [_h, _ip, _ip]),
    ("cpml_autotune", ctypes.c_int, [_h, ctypes.c_int, ctypes.c_char_p, _ip, _ip, _ip, _dp]),
    ("cpml_destroy", None, [_h]),
    ("cpml_batch_create", ctypes.c_int, [ctypes.c_int, _P(CpmlParams), _P(_h)]),
    ("cpml_batch_set_model", ctypes.c_int, [_h, ctypes.c_int, _fp, _fp, _fp]),
    ("cpml_batch_set_receivers", ctypes.c_int, [_h, ctypes.c_int, ctypes.c_int, _ip, _ip]),
    ("cpml_batch_run", ctypes.c_int, [_h]),
    ("cpml_batch_get_seismograms", ctypes.c_int, [_h, ctypes.c_int, _dp, _dp]),
    ("cpml_batch_get_field", ctypes.c_int, [_h, ctypes.c_int, ctypes.c_int, _fp]),
    ("cpml_batch_last_run_ms", ctypes.c_int, [_h, _dp]),
    ("cpml_batch_set_wait_limit", ctypes.c_int, [_h, ctypes.c_longlong]),
    ("cpml_batch_set_tuning", ctypes.c_int, [_h, ctypes.c_int, ctypes.c_int]),
    ("cpml_batch_get_tuning", ctypes.c_int, [_h, _ip, _ip]),
    ("cpml_batch_autotune", ctypes.c_int, [_h, ctypes.c_int, _ip, _ip, _dp]),
    ("cpml_batch_destroy", None, [_h]),
    ("cpml_energy3d_noalloc", ctypes.c_int, [_P(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("cpml_strerror", ctypes.c_char_p, [ctypes.c_int]),
    ("cpml_nn_gemm", ctypes.c_int, [ctypes.c_int] * 3 + [_vp, ctypes.c_int, ctypes.c_int] * 2
     + [_vp, _vp, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, _vp,
        ctypes.c_longlong, _vp]),
    ("cpml_nn_gemm_tc", ctypes.c_int, [ctypes.c_int] * 3 + [_vp, ctypes.c_int, ctypes.c_int] * 2
     + [_vp, _vp, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, _vp,
        ctypes.c_longlong, _vp]),
    ("cpml_nn_error", ctypes.c_int, [_ip]),
    ("cpml_nn_im2col", ctypes.c_int, [_vp, _vp] + [ctypes.c_int] * 4 + [_vp]),
    ("cpml_nn_col2im", ctypes.c_int, [_vp, _vp] + [ctypes.c_int] * 4 + [_vp]),
    ("cpml_nn_relu_bwd", ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_longlong, _vp]),
    ("cpml_nn_shift_rows", ctypes.c_int, [_vp, _vp, _vp, _vp] + [ctypes.c_int] * 4 + [_vp]),
    ("cpml_nn_cast", ctypes.c_int, [_vp, _vp, ctypes.c_longlong, _vp]),
    ("cpml_nn_colsum", ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp,
                                      ctypes.c_longlong, _vp]),
    ("cpml_nn_rel_l2", ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    ("cpml_nn_head_grad", ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_float,
                                         _vp]),
    ("cpml_nn_adam", ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_longlong] + [ctypes.c_float] * 4
     + [ctypes.c_int, ctypes.c_float, _vp]),
    ("cpml_write_seismograms", ctypes.c_int, [ctypes.c_char_p, _dp, _dp, _dp, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_double]),
    ("cpml_write_seismograms_su", ctypes.c_int, [ctypes.c_char_p, _dp, _dp, _dp, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_double]),
    ("cpml_write_energy", ctypes.c_int, [ctypes.c_char_p, _dp, _dp, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int]),
    ("cpml_write_pnm", ctypes.c_int, [ctypes.c_char_p, _fp, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _ip,
                                      ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int]),
]

_lib = None


class CpmlError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        name = ERR.get(status, str(status))
        msg = strerror(status) if _lib is not None else name
        super().__init__(f"{what}: CPML_ERR_{name} ({msg})" if what else f"CPML_ERR_{name} ({msg})")


def load(path: str | None = None):
    """Load libcpml.so and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"libcpml.so not built ({path}); run seismic_cpml_gb300.build.build()")
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def strerror(status: int) -> str:
    return load().cpml_strerror(status).decode()


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise CpmlError(status, what)
