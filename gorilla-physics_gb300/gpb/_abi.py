"""ctypes binding of include/gpb.h (libgpb.so).

The library is loaded from this package directory.  There is no fallback:
if libgpb.so is missing or fails to load, importing raises.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgpb.so"

# return codes / status bits / enums (include/gpb.h)
GPB_OK = 0
GPB_E_INVAL, GPB_E_NOMEM, GPB_E_CUDA, GPB_E_TIMEOUT, GPB_E_RANGE, GPB_E_STATE = -1, -2, -3, -4, -5, -6
GPB_ST_NONFINITE, GPB_ST_CHOL_FAIL, GPB_ST_COLLISION, GPB_ST_SOLVER = 1, 2, 4, 8
FIXED, REVOLUTE, PRISMATIC, FLOATING = 0, 1, 2, 3
SEMI_IMPLICIT_EULER, RUNGE_KUTTA_2, RUNGE_KUTTA_4, VELOCITY_STEPPING = 0, 1, 2, 3
FP64, MIXED, MIXED_REFINED = 0, 1, 2
ALGO_CRBA, ALGO_ABA = 0, 1
HUNT_CROSSLEY, LINEAR_SPRING_DAMPER = 0, 1
CONTROL_HOST_TAU, CONTROL_OPEN_LOOP, CONTROL_PD = 0, 1, 2
MAX_BODIES = MAX_DOF = MAX_CONTACTS = 64
MAX_HALFSPACES = 4

P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_f64 = C.POINTER(C.c_double)


class GpbModel(C.Structure):
    _fields_ = [
        ("n_instances", C.c_int64),
        ("joint_offset", P_i32),
        ("joint_type", P_i32),
        ("joint_parent", P_i32),
        ("joint_iso", P_f64),
        ("joint_axis", P_f64),
        ("joint_spring", P_f64),
        ("body_inertia", P_f64),
        ("contact_offset", P_i32),
        ("contact_body", P_i32),
        ("contact_params", P_f64),
        ("halfspace_offset", P_i32),
        ("halfspace_params", P_f64),
        ("contact_model", P_i32),
        ("joint_armature", P_f64),
        ("body_cuboid", P_f64),
    ]


class GpbControl(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("seed", C.c_uint32),
        ("resample_every", C.c_int32),
        ("sigma", C.c_double),
        ("kp", C.c_double),
        ("kd", C.c_double),
        ("tau", P_f64),
    ]


class GpbSlotClass(C.Structure):
    _fields_ = [
        ("max_bodies", C.c_int32),
        ("max_q", C.c_int32),
        ("max_v", C.c_int32),
        ("max_contacts", C.c_int32),
        ("max_halfspaces", C.c_int32),
        ("weight", C.c_double),
        ("packs", C.c_int32),
        ("chunk_steps", C.c_int32),
        ("max_cuboids", C.c_int32),
        ("planar_only", C.c_int32),
    ]


class GpbServerOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("chunk_steps", C.c_int32),
        ("hbm_budget_bytes", C.c_int64),
        ("n_classes", C.c_int32),
        ("classes", C.POINTER(GpbSlotClass)),
        ("max_admit_per_tick", C.c_int32),
        ("algorithm", C.c_int32),
    ]


class GpbRequest(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("steps", C.c_int64),
        ("integrator", C.c_int32),
        ("control", C.c_int32),
        ("seed", C.c_uint32),
        ("resample_every", C.c_int32),
        ("sigma", C.c_double),
        ("kp", C.c_double),
        ("kd", C.c_double),
        ("key", C.c_int32),
    ]


class GpbServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("pending", "active", "completed", "slots", "ticks", "pool_bytes", "steps")]


# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("gpb_abi_version", C.c_int, []),
    ("gpb_last_error", C.c_char_p, []),
    ("gpb_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("gpb_destroy", C.c_int, [C.c_void_p]),
    ("gpb_batch_create", C.c_int, [C.c_void_p, C.POINTER(GpbModel), C.POINTER(C.c_void_p)]),
    ("gpb_batch_destroy", C.c_int, [C.c_void_p]),
    ("gpb_batch_layout", C.c_int, [C.c_void_p, P_i64, P_i64, P_i64, P_i64]),
    ("gpb_set_state", C.c_int, [C.c_void_p, P_f64, P_f64]),
    ("gpb_get_state", C.c_int, [C.c_void_p, P_f64, P_f64]),
    ("gpb_dynamics", C.c_int, [C.c_void_p, P_f64, C.c_int, P_f64, P_f64]),
    ("gpb_step", C.c_int, [C.c_void_p, C.c_double, P_f64, C.c_int, C.c_int]),
    ("gpb_simulate", C.c_int, [C.c_void_p, C.c_double, C.c_int64, C.c_int64, C.c_int, C.c_int,
                               C.POINTER(GpbControl), C.c_int64, P_f64]),
    ("gpb_simulate_steps", C.c_int64, [C.c_double, C.c_double]),
    ("gpb_batch_status", C.c_int, [C.c_void_p, P_i32]),
    ("gpb_batch_clear_status", C.c_int, [C.c_void_p]),
    ("gpb_batch_steps_done", C.c_int, [C.c_void_p, P_i64]),
    ("gpb_synchronize", C.c_int, [C.c_void_p]),
    ("gpb_batch_set_launch", C.c_int, [C.c_void_p, C.c_int]),
    ("gpb_batch_set_coop", C.c_int, [C.c_void_p, C.c_int]),
    ("gpb_batch_set_algorithm", C.c_int, [C.c_void_p, C.c_int]),
    ("gpb_batch_set_gravity", C.c_int, [C.c_void_p, C.c_double]),
    ("gpb_free_velocity", C.c_int, [C.c_void_p, C.c_double, P_f64, C.c_int, P_f64]),
    ("gpb_batch_autotune", C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int, C.POINTER(GpbControl), C.c_int,
                                     P_i32, P_i32, P_i32]),
    ("gpb_batch_set_mapping", C.c_int, [C.c_void_p, C.c_int]),
    ("gpb_launch_count", C.c_int64, [C.c_void_p]),
    ("gpb_last_launch_ms", C.c_double, [C.c_void_p]),
    ("gpb_config_sizes", C.c_int, [C.c_int, C.c_int64, C.c_uint32, P_i64, P_i64, P_i64, P_i64, P_i64]),
    ("gpb_config_build", C.c_int, [C.c_int, C.c_int64, C.c_uint32, C.c_int,
                                   P_i32, P_i32, P_i32, P_f64, P_f64, P_f64, P_f64,
                                   P_i32, P_i32, P_f64, P_i32, P_f64, P_i32, P_f64, P_f64, P_f64]),
    ("gpb_open_loop_tau", C.c_double, [C.c_uint32, C.c_int64, C.c_int64, C.c_int32, C.c_double]),
    ("gpb_fma_peak", C.c_int, [C.c_int, C.c_int, C.c_int, P_f64]),
    ("gpb_cvt_peak", C.c_int, [C.c_int, P_f64]),
    ("gpb_dynamics_static", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_void_p]),
    ("gpb_collide_cuboids", C.c_int, [C.c_void_p, C.c_int64, P_f64, P_f64, P_f64, P_f64, P_i32, P_f64, P_f64]),
    ("gpb_collide_cuboids_device", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("gpb_server_plan", C.c_int, [C.POINTER(GpbServerOpts), P_i32, P_i64]),
    ("gpb_server_create", C.c_int, [C.c_void_p, C.POINTER(GpbServerOpts), C.POINTER(C.c_void_p)]),
    ("gpb_server_destroy", C.c_int, [C.c_void_p]),
    ("gpb_server_submit", C.c_int, [C.c_void_p, C.POINTER(GpbModel), C.c_int64, C.c_int64, P_f64, P_f64,
                                    P_f64, C.POINTER(GpbRequest), C.POINTER(C.c_uint64)]),
    ("gpb_server_tick", C.c_int, [C.c_void_p, P_i32]),
    ("gpb_server_completed", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int32, P_i32]),
    ("gpb_server_result", C.c_int, [C.c_void_p, C.c_uint64, P_f64, P_f64, P_i32, P_i64, P_f64]),
    ("gpb_server_forget", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int64]),
    ("gpb_server_stats_get", C.c_int, [C.c_void_p, C.POINTER(GpbServerStats)]),
]
GPB_STATIC_SCRATCH_BYTES = 16 << 20

_lib = None


def lib() -> C.CDLL:
    """Loads libgpb.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with gpb._build.build() (nvcc, sm_103a)")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class GpbError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().gpb_last_error().decode(errors="replace")
        super().__init__(f"{where} failed ({code}): {msg}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != GPB_OK:
        raise GpbError(code, where)
