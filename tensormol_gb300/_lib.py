"""ctypes binding of libtmgpu.so (the C ABI declared in include/tmgpu.h).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every entry point raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtmgpu.so")

TM_OK = 0
ERRORS = {1: "TM_E_ARG", 2: "TM_E_CUDA", 3: "TM_E_CAPACITY", 4: "TM_E_NONFINITE",
          5: "TM_E_BUDGET", 6: "TM_E_TIMEOUT", 7: "TM_E_STATE", 8: "TM_E_UNSUPPORTED"}
ERROR_CODES = {name: code for code, name in ERRORS.items()}

TM_ACT = {"relu": 0, "sigmoid_with_param": 1, "softplus": 2, "tanh": 3, "elu": 4}
TM_PREC = {"fp32": 0, "bf16": 1}
TM_F_ENERGY_ONLY = 1
TM_F_DEVICE_IO = 2
TM_F_REUSE_NLIST = 4
TM_F_REFERENCE_PERIODIC_FORCE = 8
TM_MD = {"nve": 0, "nose": 1, "nhc": 2}
TM_SERVE = {"ef": 0, "md": 1, "opt": 2}

# every symbol include/tmgpu.h declares
EXPORTS = [
    "tm_ctx_create", "tm_ctx_destroy", "tm_ctx_set_stream", "tm_ctx_stream", "tm_ctx_last_error",
    "tm_ctx_bytes_in_use", "tm_ctx_launch_count",
    "tm_model_create", "tm_model_set_layer", "tm_model_finalize", "tm_model_descriptor_width",
    "tm_model_destroy",
    "tm_system_create", "tm_system_destroy", "tm_system_natoms", "tm_system_set_positions",
    "tm_system_get_positions", "tm_system_build_nlist", "tm_system_nlist_counts",
    "tm_system_export_nlist", "tm_system_export_ee", "tm_energy_force",
    "tm_md_create", "tm_md_destroy", "tm_md_set_velocities", "tm_md_get_velocities", "tm_md_run",
    "tm_selftest_gemm", "tm_selftest_gemm_timeout", "tm_model_erfc_poly", "tm_system_descriptors", "tm_energy_force_profile",
    "tm_system_refined_units", "tm_system_layer_outputs", "tm_system_profile_layers",
    "tm_nlist_build_static",
    "tm_serve_create", "tm_serve_destroy", "tm_serve_info", "tm_serve_layout", "tm_serve_step",
    "tm_serve_read",
]


class TmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class tm_model_desc(ctypes.Structure):
    _fields_ = [
        ("n_elements", ctypes.c_int), ("elements", ctypes.c_int * 8),
        ("n_hidden", ctypes.c_int), ("hidden", ctypes.c_int * 4),
        ("activation", ctypes.c_int), ("sigmoid_alpha", ctypes.c_double),
        ("r_rc", ctypes.c_double), ("a_rc", ctypes.c_double),
        ("eta", ctypes.c_double), ("zeta", ctypes.c_double),
        ("n_r_rs", ctypes.c_int), ("n_a_rs", ctypes.c_int), ("n_a_as", ctypes.c_int),
        ("ee_cut_on", ctypes.c_double), ("ee_cut_off", ctypes.c_double),
        ("elu_width", ctypes.c_double), ("dsf_alpha", ctypes.c_double),
        ("poly_width", ctypes.c_double),
        ("add_ecc", ctypes.c_int), ("has_vdw", ctypes.c_int), ("precision", ctypes.c_int),
    ]


_LIB = None


def _declare(lib):
    P, I, D, L, U, S = (ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64,
                        ctypes.c_uint, ctypes.c_size_t)
    PP = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "tm_ctx_create": (I, [I, S, PP]),
        "tm_ctx_destroy": (I, [P]),
        "tm_ctx_set_stream": (I, [P, P]),
        "tm_ctx_stream": (P, [P]),
        "tm_ctx_last_error": (I, [P, ctypes.c_char_p, I]),
        "tm_ctx_bytes_in_use": (S, [P]),
        "tm_ctx_launch_count": (L, [P]),
        "tm_model_create": (I, [P, ctypes.POINTER(tm_model_desc), PP]),
        "tm_model_set_layer": (I, [P, I, I, I, P, P, I, I]),
        "tm_model_finalize": (I, [P]),
        "tm_model_descriptor_width": (I, [P]),
        "tm_model_destroy": (I, [P]),
        "tm_system_create": (I, [P, I, I, P, P, P, PP]),
        "tm_system_destroy": (I, [P]),
        "tm_system_natoms": (I, [P]),
        "tm_system_set_positions": (I, [P, P, I]),
        "tm_system_get_positions": (I, [P, P, I]),
        "tm_system_build_nlist": (I, [P]),
        "tm_system_nlist_counts": (I, [P, P]),
        "tm_system_export_nlist": (I, [P, P, P, P, P, I]),
        "tm_system_export_ee": (I, [P, P, L, I]),
        "tm_energy_force": (I, [P, P, U, P, P, P, P, P]),
        "tm_md_create": (I, [P, I, D, D, I, PP]),
        "tm_md_destroy": (I, [P]),
        "tm_md_set_velocities": (I, [P, P, I]),
        "tm_md_get_velocities": (I, [P, P, I]),
        "tm_md_run": (I, [P, I, D, P]),
        "tm_selftest_gemm": (I, [P, I, I, I, I, P, P, P]),
        "tm_selftest_gemm_timeout": (I, [P, I, L]),
        "tm_model_erfc_poly": (I, [P, P, P, P, P, P, P]),
        "tm_system_descriptors": (I, [P, P]),
        "tm_energy_force_profile": (I, [P, U, P]),
        "tm_system_refined_units": (I, [P, P]),
        "tm_system_layer_outputs": (I, [P, I, P]),
        "tm_system_profile_layers": (I, [P, P]),
        "tm_nlist_build_static": (I, [P, P, I, D, D, P, P, I, P, P, I, P, P]),
        "tm_serve_create": (I, [P, I, I, D, PP]),
        "tm_serve_destroy": (I, [P]),
        "tm_serve_info": (I, [P, P, P, P, P, P]),
        "tm_serve_layout": (I, [P, I, P, P, P, P, P, P]),
        "tm_serve_step": (I, [P, P, P]),
        "tm_serve_read": (I, [P, I, P, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def load(build_if_missing=False):
    """Load the in-tree library (building it first if asked)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing: run tensormol_gb300.build.build() first")
        from . import build as _b
        _b.build()
    _LIB = _declare(ctypes.CDLL(LIB_PATH))
    return _LIB


def check(ctx_ptr, rc):
    if rc != TM_OK:
        buf = ctypes.create_string_buffer(1024)
        if ctx_ptr:
            load().tm_ctx_last_error(ctx_ptr, buf, 1024)
        raise TmError(rc, buf.value.decode(errors="replace"))
