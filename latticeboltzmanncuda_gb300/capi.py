"""ctypes binding of the C ABI (include/lbm_capi.h) over liblbm_gb300.so.

Every call goes through the C ABI; there is no other code path.  If the library cannot be loaded
the import of this module's ``lib()`` raises: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblbm_gb300.so")

# enums (lbm_capi.h)
OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_UNSUPPORTED, ERR_STATE, ERR_BUDGET, ERR_TIMEOUT = range(8)
D2Q9, D3Q27_REF = 0, 1
F32, F16S, BF16S, F64 = 0, 1, 2, 3
FLUID, WALL, MOVING_WALL = 0, 1, 2
INTERNAL, REFLECTED, SOURCE = 1, 2, 4
ORDER_STREAM_COLLIDE, ORDER_CLI = 0, 1
EQ_FLOAT_FLOAT, EQ_FP64, EQ_FP32 = 0, 1, 2
OP_STREAM, OP_REFLECT, OP_COLLIDE, OP_FLOW = 1, 2, 4, 8
FORCE_REFERENCE, FORCE_MOMENTUM_EXCHANGE = 0, 1
NOALLOC_MAX_ROWS = 32768  # LBM_NOALLOC_MAX_ROWS

DTYPES = {"f32": F32, "f16s": F16S, "bf16s": BF16S, "f64": F64}
MODES = {"d2q9": D2Q9, "d3q27_ref": D3Q27_REF}

# struct LatticePoint (LatticePoint.h:9-17), 144 bytes
LATTICE_POINT = np.dtype({
    "names": ["x", "y", "z", "f", "isReflected", "isInternal", "reflections", "d_reflections"],
    "formats": [np.int32, np.int32, np.int32, (np.float32, (27,)), np.bool_, np.bool_, np.uint64, np.uint64],
    "offsets": [0, 4, 8, 12, 120, 121, 128, 136],
    "itemsize": 144,
})
# struct ReflectionValues (LatticePoint.h:3-7), 380 bytes
REFLECTION_VALUES = np.dtype([("dirs", np.int32, (14,)), ("w", np.float32, (81,))])
assert REFLECTION_VALUES.itemsize == 380

# D2Q9 population order used by the library
CX9 = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.int32)
CY9 = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.int32)
W9 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
AOS_SLOTS_D2Q9 = np.array([0, 6, 5, 1, 2, 18, 10, 7, 15], dtype=np.int32)


class Desc(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("dtype", ctypes.c_int32), ("nx", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("periodic", ctypes.c_int32),
                ("tau", ctypes.c_float), ("body_force", ctypes.c_float * 3),
                ("wall_velocity", ctypes.c_float * 3), ("order", ctypes.c_int32),
                ("force_mode", ctypes.c_int32), ("device", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class Info(ctypes.Structure):
    _fields_ = [("cells", ctypes.c_int64), ("fluid_cells", ctypes.c_int64), ("row_pitch", ctypes.c_int64),
                ("state_bytes", ctypes.c_int64), ("device_bytes", ctypes.c_int64),
                ("bytes_per_update", ctypes.c_int64), ("steps_done", ctypes.c_int64),
                ("block_threads", ctypes.c_int32), ("cells_per_thread", ctypes.c_int32),
                ("rows_per_block", ctypes.c_int32), ("tuned", ctypes.c_int32), ("l2_policy", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("device", ctypes.c_int32), ("budget_bytes", ctypes.c_int64),
                ("max_slots", ctypes.c_int32), ("round_steps", ctypes.c_int32), ("time_limit", ctypes.c_double),
                ("stream", ctypes.c_void_p)]


class Request(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("tau", ctypes.c_float),
                ("periodic", ctypes.c_int32), ("body_force", ctypes.c_float * 2),
                ("wall_velocity", ctypes.c_float * 2), ("flags", ctypes.c_void_p), ("steps", ctypes.c_int64),
                ("arrival", ctypes.c_double), ("out_rho", ctypes.c_void_p), ("out_ux", ctypes.c_void_p),
                ("out_uy", ctypes.c_void_p)]


class RequestResult(ctypes.Structure):
    _fields_ = [("admitted", ctypes.c_double), ("finished", ctypes.c_double), ("status", ctypes.c_int32),
                ("slot", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("makespan", ctypes.c_double), ("cell_updates", ctypes.c_double), ("rounds", ctypes.c_int64),
                ("peak_bytes", ctypes.c_int64), ("peak_slots", ctypes.c_int32), ("rejected", ctypes.c_int32),
                ("round_seconds", ctypes.c_double), ("tile_shape", ctypes.c_int32 * 3), ("tunings", ctypes.c_int32)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_int64), ("faces", ctypes.c_int64), ("triangle_mesh", ctypes.c_int32),
                ("closed", ctypes.c_int32), ("valid", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("bbox_min", ctypes.c_float * 3), ("bbox_max", ctypes.c_float * 3)]


# exported symbols and their signatures: (name, restype, argtypes)
_P, _I32, _I64, _U64, _F = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_float
_S = ctypes.c_int
SIGNATURES = [
    ("lbm_desc_init", None, [_P]),
    ("lbm_create", _S, [_P, _P]),
    ("lbm_destroy", _S, [_P]),
    ("lbm_last_error", ctypes.c_char_p, [_P]),
    ("lbm_status_string", ctypes.c_char_p, [_S]),
    ("lbm_get_info", _S, [_P, _P]),
    ("lbm_get_stream", _S, [_P, _P]),
    ("lbm_synchronize", _S, [_P]),
    ("lbm_set_params", _S, [_P, _F, _P, _P]),
    ("lbm_set_flags", _S, [_P, _P]),
    ("lbm_get_flags", _S, [_P, _P]),
    ("lbm_init_equilibrium", _S, [_P, _P, _P, _P]),
    ("lbm_load_populations", _S, [_P, _P, _I32]),
    ("lbm_retrieve_populations", _S, [_P, _P, _I32]),
    ("lbm_load_aos", _S, [_P, _P, _I64]),
    ("lbm_retrieve_aos", _S, [_P, _P, _I64]),
    ("lbm_set_reflection_tables", _S, [_P, _I64, _P, _P]),
    ("lbm_set_flow", _S, [_P, _P, _P]),
    ("lbm_set_force", _S, [_P, _P, _I32]),
    ("lbm_get_force", _S, [_P, _P]),
    ("lbm_step", _S, [_P, _I32]),
    ("lbm_apply", _S, [_P, _I32]),
    ("lbm_set_order", _S, [_P, _I32]),
    ("lbm_set_equilibrium_evaluation", _S, [_P, _I32]),
    ("lbm_d3q27_equilibrium_selftest", _S, [_I64, _U64, _I32, _P]),
    ("lbm_d3q27_division_check", _S, [_F, _I32, _P]),
    ("lbm_set_force_accumulation", _S, [_P, _I32]),
    ("lbm_force_accumulation", _I32, [_P]),
    ("lbm_step_force_series", _S, [_P, _I32, _P]),
    ("lbm_autotune", _S, [_P, _I32]),
    ("lbm_set_launch", _S, [_P, _I32, _I32, _I32, _I32]),
    ("lbm_set_sweep_alternation", _S, [_P, _I32]),
    ("lbm_set_pipeline_wait", _S, [_P, _I64, _I32]),
    ("lbm_save", _S, [_P, ctypes.c_char_p]),
    ("lbm_load", _S, [_P, ctypes.c_char_p]),
    ("lbm_checkpoint_desc", _S, [ctypes.c_char_p, _P]),
    ("lbm_moments", _S, [_P, _P, _P, _P, _P]),
    ("lbm_conservation", _S, [_P, _P]),
    ("lbm_batch_create", _S, [_I32, _I32, _P, _P]),
    ("lbm_batch_destroy", _S, [_P]),
    ("lbm_batch_last_error", ctypes.c_char_p, [_P]),
    ("lbm_batch_slot_bytes", _I64, [_I32, _I32, _I32]),
    ("lbm_batch_add", _S, [_P, _P, _P, _P]),
    ("lbm_batch_remove", _S, [_P, _I32]),
    ("lbm_batch_step", _S, [_P, _I32]),
    ("lbm_batch_autotune", _S, [_P]),
    ("lbm_batch_tunings", _S, [_P, _P]),
    ("lbm_batch_set_launch", _S, [_P, _I32, _I32, _I32]),
    ("lbm_batch_synchronize", _S, [_P]),
    ("lbm_batch_set_persistent", _S, [_P, _I32, _I64, _I32]),
    ("lbm_batch_get_stream", _S, [_P, _P]),
    ("lbm_batch_info", _S, [_P, _P]),
    ("lbm_batch_slot_steps", _S, [_P, _I32, _P]),
    ("lbm_batch_set_slot_steps", _S, [_P, _I32, _I64]),
    ("lbm_batch_moments", _S, [_P, _I32, _P, _P, _P]),
    ("lbm_batch_moments_async", _S, [_P, _I32, _P]),
    ("lbm_batch_collect", _S, [_P, _I64, _I32, _P, _P, _P, _P]),
    ("lbm_batch_load_populations", _S, [_P, _I32, _P, _I32]),
    ("lbm_batch_retrieve_populations", _S, [_P, _I32, _P, _I32]),
    ("lbm_server_config_init", None, [_P]),
    ("lbm_server_create", _S, [_P, _P]),
    ("lbm_server_destroy", _S, [_P]),
    ("lbm_server_last_error", ctypes.c_char_p, [_P]),
    ("lbm_server_run", _S, [_P, _P, _I64, _P, _P]),
    ("lbm_d2q9_conservation_noalloc", _S, [_P, _I32, _P, _I32, _I32, _I64, _P, _P]),
    ("lbm_gen_channel", _S, [_I32, _I32, _I32, _F, _F, _U64, _P, _P]),
    ("lbm_gen_cavity", _S, [_I32, _I32, _P]),
    ("lbm_gen_disks_fraction", _S, [_I32, _I32, _F, _F, _F, _U64, _P, _P]),
    ("lbm_mesh_load_obj", _S, [ctypes.c_char_p, _P]),
    ("lbm_mesh_create", _S, [_P, _I64, _P, _I64, _P, _P]),
    ("lbm_mesh_destroy", None, [_P]),
    ("lbm_mesh_get_info", _S, [_P, _P]),
    ("lbm_mesh_point_inside", _S, [_P, _P, _P]),
    ("lbm_mesh_reflection_vector", _S, [_P, _P, _P, _P]),
    ("lbm_rotate_vector", None, [_P, _P, _F, _P]),
    ("lbm_distribute_vector", None, [_P, _P, _P]),
    ("lbm_mesh_rasterize", _S, [_P, _I32, _I32, _I32, _F, _P, _P]),
    ("lbm_mesh_reflection_tables", _S, [_P, _I32, _I32, _I32, _F, _P, _I64, _P, _P, _P]),
]

_lib = None


class LBMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def lib(build: bool = True):
    """Load liblbm_gb300.so (building it with nvcc first when it is missing or stale)."""
    global _lib
    if _lib is None:
        if build:
            from . import build as _b
            _b.build()
        if not os.path.exists(LIB_PATH):
            raise LBMError(ERR_STATE, f"{LIB_PATH} is missing: build it with python -m latticeboltzmanncuda_gb300.build")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def check(status, ctx=None):
    if status != OK:
        msg = lib().lbm_last_error(ctx)
        raise LBMError(status, (msg or b"").decode() or lib().lbm_status_string(status).decode())


def last_thread_error() -> str:
    return (lib().lbm_last_error(None) or b"").decode()
