"""ctypes binding of the C-ABI library ``libdpgb.so`` (include/dpgb.h).

There is no CPU fallback: if the library is missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)

MAX_TYPES = 8
MAX_LAYERS = 6


class DpgbError(RuntimeError):
    """Raised when a dpgb entry point returns a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"dpgb error {code}: {msg}")
        self.code = code


class SeADesc(C.Structure):
    """dpgb_se_a_desc of include/dpgb.h."""

    _fields_ = [
        ("ntypes", C.c_int),
        ("sel", C.c_int * MAX_TYPES),
        ("rcut", C.c_double),
        ("rcut_smth", C.c_double),
        ("type_one_side", C.c_int),
        ("n_emb", C.c_int),
        ("emb_neuron", C.c_int * MAX_LAYERS),
        ("axis_neuron", C.c_int),
        ("n_fit", C.c_int),
        ("fit_neuron", C.c_int * MAX_LAYERS),
        ("dim_descrpt", C.c_int),
        ("davg", _DP),
        ("dstd", _DP),
        ("emb_w", (_DP * MAX_LAYERS) * (MAX_TYPES * MAX_TYPES)),
        ("emb_b", (_DP * MAX_LAYERS) * (MAX_TYPES * MAX_TYPES)),
        ("emb_idt", (_DP * MAX_LAYERS) * (MAX_TYPES * MAX_TYPES)),
        ("fit_w", (_DP * (MAX_LAYERS + 1)) * MAX_TYPES),
        ("fit_b", (_DP * (MAX_LAYERS + 1)) * MAX_TYPES),
        ("fit_idt", (_DP * (MAX_LAYERS + 1)) * MAX_TYPES),
        ("atom_ener_bias", _DP),
        ("pair_mask", _IP),
        ("table", _DP * (MAX_TYPES * MAX_TYPES)),
        ("table_info", (C.c_double * 6) * (MAX_TYPES * MAX_TYPES)),
        ("compressed", C.c_int),
    ]


class SeABlock(C.Structure):
    """dpgb_se_a_block of include/dpgb.h."""

    _fields_ = [
        ("ntypes", C.c_int),
        ("sel", C.c_int * MAX_TYPES),
        ("type_one_side", C.c_int),
        ("n_layer", C.c_int),
        ("neuron", C.c_int * MAX_LAYERS),
        ("axis_neuron", C.c_int),
        ("resnet_dt", C.c_int),
        ("pair_keep", C.c_int * ((MAX_TYPES + 1) * (MAX_TYPES + 1))),
    ]


# name -> argtypes (all return int unless listed in _RESTYPE)
_SIGS = {
    "dpgb_last_error": [],
    "dpgb_version": [],
    "dpgb_tabulate_fusion_se_a_f64": [_P, _P, _DP, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_tabulate_fusion_se_a_f32": [_P, _P, _FP, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_tabulate_fusion_se_a_grad_f64": [_P, _P, _P, _DP, _P, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_tabulate_fusion_se_a_grad_f32": [_P, _P, _P, _FP, _P, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_tabulate_fusion_se_a_grad_grad_f64": [_P, _P, _DP, _P, _P, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_tabulate_fusion_se_a_grad_grad_f32": [_P, _P, _FP, _P, _P, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_format_nlist_a": [_P, _P, _P, _P, _P, _I, _I, _I, _D, _IP, _I, _IP, _P],
    "dpgb_build_nlist_pt": [_P, _P, _P, _I, _DP, _IP, _I, _D, _IP, _I, _P],
    "dpgb_normalize_coord": [_P, _P, _I, _DP, _P],
    "dpgb_extend_coord": [_P, _P, _P, _P, _P, _I, _DP, _IP, _I, _P],
    "dpgb_prod_env_mat_a_f64": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _P, _P, _I, _I, _D, _D, _IP, _I, _P],
    "dpgb_env_mat_pt_f64": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _P],
    "dpgb_env_mat_pt2_f64": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D, _P],
    "dpgb_env_mat_pt2_f32": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D, _P],
    "dpgb_env_mat_pt_bwd_f64": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D, _P],
    "dpgb_env_mat_pt_bwd_f32": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _D, _D, _P],
    "dpgb_env_mat_pt_bwd_bwd_f64": [_P] * 12 + [_I, _I, _I, _I, _D, _D, _D, _P],
    "dpgb_env_mat_pt_bwd_bwd_f32": [_P] * 12 + [_I, _I, _I, _I, _D, _D, _D, _P],
    "dpgb_se_a_table_rows": [_D, _D, _D, _D, _D],
    "dpgb_se_a_table_build_f64": [_P, _P, _P, _I, _D, _D, _D, _D, _D, _P],
    "dpgb_se_a_block_param_count": [_P],
    "dpgb_se_a_block_workspace_bytes": [_P, _I, _I, _I],
    "dpgb_se_a_block_fwd_f64": [_P, _P, _P, _P, _P, _I, _I, _I, _P, _P, _P],
    "dpgb_se_a_block_fwd_f32": [_P, _P, _P, _P, _P, _I, _I, _I, _P, _P, _P],
    "dpgb_se_a_block_bwd_f64": [_P, _P, _P, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, C.c_size_t, _P],
    "dpgb_se_a_block_bwd_f32": [_P, _P, _P, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, C.c_size_t, _P],
    "dpgb_se_a_block_bwd_bwd_f64": [_P, _P, _P, _P, _P, _I, _I, _I] + [_P] * 8 + [C.c_size_t, _P],
    "dpgb_se_a_block_bwd_bwd_f32": [_P, _P, _P, _P, _P, _I, _I, _I] + [_P] * 8 + [C.c_size_t, _P],
    "dpgb_prod_force_a_f64": [_P, _P, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_prod_virial_a_f64": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _P],
    "dpgb_prod_force_a_f64_noalloc": [_P, _P, _P, _P, _I, _I, _I, _I, _P],
    "dpgb_prod_force_grad_a_f64": [_P, _P, _P, _P, _I, _I, _I, _P],
    "dpgb_prod_virial_grad_a_f64": [_P, _P, _P, _P, _P, _I, _I, _P],
    "dpgb_tc_gemm_bf16": [_P, _P, _P, _I, _I, _I, _P],
    "dpgb_deeppot_new": [C.POINTER(SeADesc), _I],
    "dpgb_deeppot_delete": [_P],
    "dpgb_deeppot_check_ok": [_P],
    "dpgb_deeppot_compute": [_P, _I, _I, _DP, _IP, _DP, _DP, _DP, _DP, _DP, _DP],
    "dpgb_deeppot_compute_device": [_P, _I, _I, _P, _IP, _DP, _P, _P, _P, _P, _P, _P],
    "dpgb_deeppot_compute_nlist": [_P, _I, _I, _DP, _IP, _DP, _I, _IP, _IP, C.POINTER(_IP), _I, _DP, _DP, _DP,
                                   _DP, _DP],
    "dpgb_batch_new": [_P, _I, _IP, _IP, _DP],
    "dpgb_batch_delete": [_P],
    "dpgb_batch_natoms": [_P],
    "dpgb_batch_compute_device": [_P, _P, _P, _P, _P, _P, _I],
    "dpgb_batch_compute": [_P, _DP, _DP, _DP, _DP, _I],
    "dpgb_batch_buckets": [_P, _IP, _IP],
    "dpgb_extend_input_and_build_nlist": [_P, _P, _P, _P, _P, _P, _I, _I, _DP, _IP, _I, _D, _IP, _I, _P],
    "dpgb_deeppot_descrpt_fwd": [_P, _I, _I, _I, _P, _P, _IP, _P, _P, _P, C.POINTER(C.c_ulonglong), _P],
    "dpgb_deeppot_descrpt_bwd": [_P, C.c_ulonglong, _P, _P, _P],
    "dpgb_batch_set_tiles": [_P, _IP],
    "dpgb_batch_get_tiles": [_P, _IP],
    "dpgb_deeppot_last_launches": [_P],
    "dpgb_deeppot_last_nlist": [_P, _IP, _IP, _DP, _DP],
    "dpgb_selftest_wait_timeout": [_D, _P],
    "dpgb_model_file_open": [C.c_char_p, C.c_char_p, C.c_size_t],
    "dpgb_model_file_close": [_P],
    "dpgb_model_file_desc": [_P],
    "dpgb_model_file_type_map": [_P],
    "dpgb_model_file_config": [_P],
    "dpgb_model_file_tensor": [_P, C.c_char_p, _DP, C.c_longlong, C.POINTER(C.c_longlong), _IP],
    "dpgb_deeppot_set_skin": [_P, _D, _I],
    "dpgb_deeppot_set_graph": [_P, _I],
    "dpgb_deeppot_check_status": [_P, _P],
    "dpgb_deeppot_set_profiling": [_P, _I],
    "dpgb_deeppot_collect_stages": [_P],
    "dpgb_deeppot_stage_times": [_P, _DP, _IP],
}
STAGES = ["nlist", "transpose", "desc_fwd", "fitting", "desc_bwd", "reduce"]
_RESTYPE = {
    "dpgb_last_error": C.c_char_p,
    "dpgb_version": C.c_char_p,
    "dpgb_deeppot_new": _P,
    "dpgb_batch_new": _P,
    "dpgb_model_file_open": _P,
    "dpgb_model_file_close": None,
    "dpgb_model_file_desc": _P,
    "dpgb_model_file_type_map": C.c_char_p,
    "dpgb_model_file_config": C.c_char_p,
    "dpgb_model_file_tensor": C.c_longlong,
    "dpgb_batch_delete": None,
    "dpgb_deeppot_delete": None,
    "dpgb_deeppot_check_ok": C.c_char_p,
    "dpgb_se_a_block_param_count": C.c_longlong,
    "dpgb_se_a_block_workspace_bytes": C.c_size_t,
}
EXPORTED = sorted(_SIGS)

_lock = threading.Lock()
_handle = None


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """The loaded library.  Builds it in-tree when missing (nvcc required)."""
    global _handle
    with _lock:
        if _handle is None:
            path = lib_path()
            if build_if_missing and (not os.path.exists(path) or _build.needs_build()):
                _build.build()
            if not os.path.exists(path):
                raise ImportError(f"dpgb CUDA library not found at {path}")
            h = C.CDLL(path)
            for name, args in _SIGS.items():
                fn = getattr(h, name)
                fn.argtypes = args
                fn.restype = _RESTYPE.get(name, C.c_int)
            _handle = h
    return _handle


def check(rc: int) -> None:
    if rc != 0:
        raise DpgbError(rc, lib().dpgb_last_error().decode())


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
