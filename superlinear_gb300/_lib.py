"""ctypes loader for the in-tree CUDA engine ``_build/libsus2g.so`` (C ABI of include/sus2g.h).

There is no CPU fallback: if the library is missing the import of any engine entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsus2g.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "sus2g.h")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "sus2g_last_error": (ctypes.c_char_p, []),
    "sus2g_abi_version": (ctypes.c_int, []),
    "sus2g_model_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "sus2g_model_free": (None, [_vp]),
    "sus2g_model_dims": (ctypes.c_int, [_vp, _ip]),
    "sus2g_model_cutoff": (ctypes.c_int, [_vp, _dp]),
    "sus2g_model_param_count": (ctypes.c_int, [_vp, _ip]),
    "sus2g_model_get_params": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
    "sus2g_model_set_params": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
    "sus2g_model_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "sus2g_engine_create": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]),
    "sus2g_engine_free": (None, [_vp]),
    "sus2g_engine_update_params": (ctypes.c_int, [_vp, _vp]),
    "sus2g_engine_set_stream": (ctypes.c_int, [_vp, _vp]),
    "sus2g_engine_take_launch_count": (ctypes.c_int, [_vp, _ip]),
    "sus2g_engine_edge_count": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "sus2g_engine_copy_edges": (ctypes.c_int, [_vp, ctypes.c_longlong, _ip, _ip, _dp,
                                               ctypes.POINTER(ctypes.c_longlong)]),
    "sus2g_engine_set_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_engine_set_step_graph": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_engine_set_pdl": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_engine_set_moment_mma": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_engine_set_static_split": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_engine_set_grad_split": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_engine_pass_shape": (ctypes.c_int, [_vp, ctypes.c_int, _ip]),
    "sus2g_engine_set_pass_shape": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_int]),
    "sus2g_engine_autotune": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp]),
    "sus2g_model_get_scaling": (ctypes.c_int, [_vp, _dp]),
    "sus2g_model_set_scaling": (ctypes.c_int, [_vp, ctypes.c_double]),
    "sus2g_trainer_rescale": (ctypes.c_int, [_vp, _dp, _dp, _ip]),
    "sus2g_engine_take_stage_times": (ctypes.c_int, [_vp, _dp, _ip]),
    # per-step entry points: raw addresses (numpy's data_as costs ~3 us per array per call)
    "sus2g_calc_efs_host": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sus2g_calc_efs_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sus2g_efs_edges_host": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int, _ip, _ip, _dp, _dp,
                                            _dp, _dp, _dp]),
    "sus2g_calc_descriptors_host": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp, _ip, _dp]),
    "sus2g_efs_combination_grad_host": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp, _ip, _dp, _dp, _dp, _dp]),
    "sus2g_efs_combination_grad_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sus2g_static_efs_noalloc": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp,
                                                ctypes.c_longlong, _vp, _vp, _vp, _vp]),
    "sus2g_engine_comm_width": (ctypes.c_int, [_vp, _ip]),
    "sus2g_stage_begin": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int, _ip, _ip, _dp]),
    "sus2g_stage_pack_forward": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp]),
    "sus2g_stage_unpack_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    "sus2g_stage_outer": (ctypes.c_int, [_vp]),
    "sus2g_stage_pack_reverse": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    "sus2g_stage_add_reverse": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp]),
    "sus2g_stage_finish": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "sus2g_trainer_create": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp, _ip, _dp, _dp, _dp, _ip,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, ctypes.POINTER(_vp)]),
    "sus2g_trainer_free": (None, [_vp]),
    "sus2g_trainer_loss_grad": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "sus2g_trainer_set_graph": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_trainer_metrics": (ctypes.c_int, [_vp, _dp, _dp]),
    "sus2g_trainer_train_linear": (ctypes.c_int, [_vp, _dp]),
    "sus2g_trainer_bfgs": (ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_double, _dp, _ip]),
    "sus2g_trainer_set_inv_hess_diagonal": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
    "sus2g_trainer_set_line_search": (ctypes.c_int, [_vp, ctypes.c_int]),
    "sus2g_trainer_bfgs_trials": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _ip, _ip]),
}

_lib = None


def header_functions(path: str = HEADER):
    """Function names declared in include/sus2g.h."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sus2g_[a-z0-9_]+)\s*\(", text)))


def load():
    """Load (once) and return the engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"CUDA engine library not built: {LIB_PATH} (run superlinear_gb300.build.build())")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class Sus2Error(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def check(rc: int) -> None:
    if rc:
        raise Sus2Error(rc, load().sus2g_last_error().decode())
