"""ctypes binding of libbgk2d_gb300.so (declarations in include/bgk2d_gb300.h).

The library is built in-tree by bgk2d_gpu_gb300/build.py.  There is no CPU fallback: when the
shared library is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

I32 = ctypes.c_int32
I64 = ctypes.c_int64
F64 = ctypes.c_double
F32 = ctypes.c_float
VP = ctypes.c_void_p

# status codes
OK, E_INVALID, E_NOMEM, E_CUDA, E_UNSUPPORTED, E_NUMERIC, E_CANCELLED, E_TIMEOUT, E_NOTFOUND, E_TOOLARGE = range(10)
STATUS_NAMES = {0: "OK", 1: "BGK_E_INVALID", 2: "BGK_E_NOMEM", 3: "BGK_E_CUDA", 4: "BGK_E_UNSUPPORTED",
                5: "BGK_E_NUMERIC", 6: "BGK_E_CANCELLED", 7: "BGK_E_TIMEOUT", 8: "BGK_E_NOTFOUND",
                9: "BGK_E_TOOLARGE"}

STORE = {"f32": 0, "f64": 1, "f16": 2, "bf16": 3}
COMPUTE = {"f32": 0, "f64": 1}
SCHEME = {"pingpong": 0, "aa": 1, "original": 2}
CASE = {"LDC": 0, "TGV": 1, "POF": 2, "VKS": 3, "COU": 4, "BFS": 5, "MYV": 6, "CUSTOM": 9}
FACE = {"wall": 0, "periodic": 1, "inflow": 2, "outflow_eq": 3, "outflow_zg": 4}
OBS = {None: 0, "none": 0, "circle": 1, "square": 2, "half_circle": 3, "mask": 4}
INIT = {"rest": 0, "tgv_ref": 1, "tgv": 2}


class CaseDesc(ctypes.Structure):
    _fields_ = [
        ("lx", I32), ("ly", I32), ("ipad", I32), ("jpad", I32),
        ("storage", I32), ("compute", I32), ("scheme", I32), ("tcase", I32),
        ("faces", I32 * 4), ("wall_u", (F64 * 2) * 4),
        ("svisc", F64), ("u0", F64), ("omega", F64), ("u_inflow", F64),
        ("inflow_profile", I32), ("obstacle", I32), ("radius", I32),
        ("obs_icoord", I32), ("obs_jcoord", I32),
        ("obs_mask", ctypes.POINTER(I32)),
        ("init_v", I32), ("tgv_u0", F64), ("device", I32), ("les", I32), ("cte_s", F64), ("trick1", I32),
        ("noshift", I32), ("force_y", I32),
        ("reserved", I32 * 1),
    ]


REQ = {"ldc": 0, "cylinder": 1, "tgv": 2}


class Request(ctypes.Structure):
    _fields_ = [("kind", I32), ("n", I32), ("re", F64), ("u", F64), ("storage", I32), ("max_steps", I32),
                ("tol", F64), ("check_every", I32), ("keep_fields", I32)]


class Result(ctypes.Structure):
    _fields_ = [("id", I64), ("status", I32), ("steps", I32), ("lx", I32), ("ly", I32), ("residual", F64),
                ("diagno", F64 * 4), ("draglift", F64 * 2), ("t_submit", F64), ("t_admit", F64), ("t_done", F64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", I32), ("max_slots", I32), ("hbm_budget", I64), ("chunk_steps", I32), ("tile_cfg", I32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", I64), ("admitted", I64), ("completed", I64), ("failed", I64),
                ("cell_updates", I64), ("busy_s", F64), ("wall_s", F64), ("glups", F64), ("p50_s", F64),
                ("p99_s", F64), ("mean_queue_s", F64), ("peak_resident", I32), ("launches", I64),
                ("rounds", I64), ("mean_round_steps", F64)]


class BgkError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")


_LIB = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it in-tree if needed).  Raises when it is unavailable."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise BgkError(E_CUDA, f"{path} is not built; run bgk2d_gpu_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    H = VP
    P = ctypes.POINTER
    sig = {
        "bgk_default_desc": (I32, [P(CaseDesc)]),
        "bgk_create": (I32, [P(CaseDesc), P(H)]),
        "bgk_destroy": (I32, [H]),
        "bgk_upload": (I32, [H, P(VP), I64]),
        "bgk_download": (I32, [H, P(VP), I64]),
        "bgk_advance_host": (I32, [H, P(VP), P(VP), I64, I32]),
        "bgk_boundaries": (I32, [H]),
        "bgk_propagation": (I32, [H]),
        "bgk_collision": (I32, [H, I32]),
        "bgk_step": (I32, [H, I32]),
        "bgk_step_timed": (I32, [H, I32, P(ctypes.c_float)]),
        "bgk_sync": (I32, [H]),
        "bgk_diagno": (I32, [H, I32, P(F64)]),
        "bgk_draglift": (I32, [H, P(F64)]),
        "bgk_draglift_reference": (I32, [H, P(F64)]),
        "bgk_residual": (I32, [H, P(F64)]),
        "bgk_fields": (I32, [H, P(F64), P(F64), P(F64)]),
        "bgk_vtk_fields": (I32, [H, P(F32), P(F32), P(F32), P(F32), P(F32)]),
        "bgk_prof_i": (I32, [H, I32, P(F64), P(F64), P(F64)]),
        "bgk_prof_j": (I32, [H, I32, P(F64), P(F64), P(F64)]),
        "bgk_varm": (I32, [H, P(F64), P(F64), P(F64)]),
        "bgk_probe": (I32, [H, I32, I32, P(F64)]),
        "bgk_get_obs": (I32, [H, P(I32), P(I32)]),
        "bgk_get_scalars": (I32, [H, P(F64), P(I64)]),
        "bgk_footprint": (I32, [H, P(I64), P(I32)]),
        "bgk_launch_count": (I32, [H, P(I64)]),
        "bgk_last_error": (I32, [H, ctypes.c_char_p, ctypes.c_size_t]),
        "bgk_version": (ctypes.c_char_p, []),
        "bgk_set_tile": (I32, [H, I32]),
        "bgk_tune": (I32, [H, I32, P(I32), P(I32)]),
        "bgk_set_prefetch": (I32, [H, I32]),
        "bgk_get_prefetch": (I32, [H, P(I32)]),
        "bgk_batch_create": (I32, [I32, I32, I32, P(VP)]),
        "bgk_batch_destroy": (I32, [VP]),
        "bgk_batch_add": (I32, [VP, H]),
        "bgk_batch_remove": (I32, [VP, H]),
        "bgk_batch_size": (I32, [VP, P(I32), P(I64)]),
        "bgk_batch_step": (I32, [VP, I32]),
        "bgk_batch_step_timed": (I32, [VP, I32, P(ctypes.c_float)]),
        "bgk_batch_sync": (I32, [VP]),
        "bgk_batch_set_config": (I32, [VP, I32, I32, I32]),
        "bgk_batch_set_prefetch": (I32, [VP, I32]),
        "bgk_batch_get_config": (I32, [VP, P(I32)]),
        "bgk_batch_tune": (I32, [VP, I32, P(I32)]),
        "bgk_batch_launch_count": (I32, [VP, P(I64)]),
        "bgk_server_create": (I32, [P(ServerConfig), P(VP)]),
        "bgk_server_destroy": (I32, [VP]),
        "bgk_server_submit": (I32, [VP, P(Request), P(I64)]),
        "bgk_server_poll": (I32, [VP, P(Result), I32, P(I32)]),
        "bgk_server_drain": (I32, [VP, F64]),
        "bgk_server_fields": (I32, [VP, I64, P(F64), P(F64), P(F64), I64]),
        "bgk_server_get_stats": (I32, [VP, P(ServerStats)]),
        "bgk_diagno_noalloc": (I32, [P(VP), I64, I32, I32, I32, P(F64)]),
        "bgk_peak_fp64": (I32, [I32, P(F64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def exported_symbols():
    """Names declared in include/bgk2d_gb300.h (the C ABI surface)."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "bgk2d_gb300.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(bgk_\w+)\s*\(", text, flags=re.M)))
