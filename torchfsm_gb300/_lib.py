"""ctypes binding of the C ABI in ``include/torchfsm_gb300.h``.

The library is loaded on first use. When it is missing, or the tensors are
not on a CUDA device, calls raise: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libtorchfsm_gb300.so")

FSM_OK = 0
FSM_ERR_INVALID = 1
FSM_ERR_UNSUPPORTED = 2
FSM_ERR_CUDA = 3
FSM_ERR_OOM = 4
FSM_ERR_NONFINITE = 5
FSM_ERR_TIMEOUT = 6

FSM_NL_NONE = 0
FSM_NL_CONVECTION = 1
FSM_NL_VORTICITY = 2
FSM_NL_KS = 3
FSM_NL_LERAY = 4

FSM_FLAG_REMOVE_MEAN = 1

FSM_STATIC_SCRATCH_BYTES = 32 * 1024 * 1024  # include/torchfsm_gb300.h

FSM_ETDRK0 = 0
FSM_ETDRK1 = 1
FSM_ETDRK2 = 2
FSM_SETDRK1 = 11
FSM_SETDRK2 = 12
FSM_SETDRK3 = 13
FSM_SETDRK4 = 14
FSM_RK_EULER = 21
FSM_RK_MIDPOINT = 22
FSM_RK_HEUN12 = 23
FSM_RK_RALSTON12 = 24
FSM_RK_BOGACKI_SHAMPINE23 = 25
FSM_RK4 = 26
FSM_RK4_38RULE = 27
FSM_RK_DORPI45 = 28
FSM_RK_FEHLBERG45 = 29
FSM_RK_CASHKARP45 = 30
FSM_APPLY = 40

FSM_SERVE_GRAPHS = 1
FSM_SERVE_UNKNOWN = -1
FSM_SERVE_WAITING = 0
FSM_SERVE_ACTIVE = 1
FSM_SERVE_DONE = 2
FSM_SERVE_NSTATS = 10

# Every symbol the header declares; tests check that the library exports them.
EXPORTS = (
    "fsm_plan_create",
    "fsm_plan_destroy",
    "fsm_plan_set_batch_dt",
    "fsm_plan_move_batch",
    "fsm_plan_tables",
    "fsm_plan_workspace_bytes",
    "fsm_plan_launch_count",
    "fsm_integrate",
    "fsm_integrate_profiled",
    "fsm_integrate_static",
    "fsm_rfftn",
    "fsm_irfftn",
    "fsm_nonfinite_flags",
    "fsm_adj_accumulate",
    "fsm_adj_vjp_products",
    "fsm_adj_vjp_combine",
    "fsm_step_adjoint_workspace_bytes",
    "fsm_step_adjoint",
    "fsm_serve_workspace_bytes",
    "fsm_serve_create",
    "fsm_serve_submit",
    "fsm_serve_tick",
    "fsm_serve_poll",
    "fsm_serve_cancel",
    "fsm_serve_request_status",
    "fsm_serve_stats",
    "fsm_serve_destroy",
    "fsm_serve_group_create",
    "fsm_serve_group_tick",
    "fsm_serve_group_poll",
    "fsm_serve_group_stats",
    "fsm_serve_group_destroy",
    "fsm_last_error",
    "fsm_abi_version",
)


class FsmError(RuntimeError):
    """A non-zero status from the library."""

    def __init__(self, code: int, message: str):
        super().__init__(f"torchfsm_gb300 error {code}: {message}")
        self.code = code


class UnsupportedProgram(FsmError):
    """No fused kernel exists for this program or mesh."""


class FsmMeshDesc(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("n", ctypes.c_int32 * 3), ("length", ctypes.c_double * 3)]


class FsmProgramDesc(ctypes.Structure):
    _fields_ = [
        ("n_channel", ctypes.c_int32),
        ("nonlinear", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("nonlinear_coef", ctypes.c_double),
        ("keep", ctypes.c_void_p * 3),
        ("n_integration_points", ctypes.c_int32),
        ("integration_radius", ctypes.c_double),
        ("linear_coef", ctypes.c_void_p),
        ("lin_batch", ctypes.c_int32),
        ("lin_channel", ctypes.c_int32),
        ("source", ctypes.c_void_p),
        ("src_batch", ctypes.c_int32),
        ("table_batch", ctypes.c_int32),
    ]


_lock = threading.Lock()
_lib: Optional[ctypes.CDLL] = None


def library_path() -> str:
    return LIB_PATH


def load(path: Optional[str] = None) -> ctypes.CDLL:
    """Load (once) and return the library; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"torchfsm_gb300 CUDA library not found at {p}; build it with "
                "`python -m torchfsm_gb300.build` (nvcc, sm_103a)"
            )
        lib = ctypes.CDLL(p)
        vp, i32, i64, sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
        lib.fsm_plan_create.argtypes = [ctypes.POINTER(FsmMeshDesc), ctypes.POINTER(FsmProgramDesc), ctypes.c_double, vp,
                                        ctypes.POINTER(vp)]
        lib.fsm_plan_destroy.argtypes = [vp]
        lib.fsm_plan_set_batch_dt.argtypes = [vp, i32, ctypes.c_double, vp]
        lib.fsm_plan_move_batch.argtypes = [vp, i32, i32, vp]
        lib.fsm_plan_tables.argtypes = [vp, vp, sz, ctypes.POINTER(i32), ctypes.POINTER(i64), vp]
        lib.fsm_plan_workspace_bytes.argtypes = [vp, i32, i32, ctypes.POINTER(sz)]
        lib.fsm_plan_launch_count.argtypes = [vp, i32, i32, ctypes.POINTER(i64)]
        lib.fsm_integrate.argtypes = [vp, i32, vp, i32, vp, vp, i32, vp, sz, vp]
        lib.fsm_integrate_profiled.argtypes = [vp, i32, vp, i32, vp, sz, vp, ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(i64)]
        lib.fsm_integrate_static.argtypes = [vp, i32, vp, i32, vp]
        lib.fsm_rfftn.argtypes = [vp, i32, vp, vp, vp]
        lib.fsm_irfftn.argtypes = [vp, i32, vp, vp, vp]
        lib.fsm_nonfinite_flags.argtypes = [vp, i32, vp, vp, vp]
        lib.fsm_adj_accumulate.argtypes = [i64, vp, vp, vp, vp]
        lib.fsm_adj_vjp_products.argtypes = [i32, i32, i64, ctypes.c_float, vp, vp, vp, vp, vp, vp, vp, vp]
        lib.fsm_adj_vjp_combine.argtypes = [i32, i32, i64, vp, vp, vp, vp, vp, vp, vp, vp]
        lib.fsm_step_adjoint_workspace_bytes.argtypes = [vp, i32, ctypes.POINTER(sz)]
        lib.fsm_step_adjoint.argtypes = [vp, i32, vp, vp, vp, vp, vp, sz, vp]
        pi32, pi64 = ctypes.POINTER(i32), ctypes.POINTER(i64)
        lib.fsm_serve_workspace_bytes.argtypes = [vp, i32, i32, ctypes.POINTER(sz)]
        lib.fsm_serve_create.argtypes = [vp, i32, i32, vp, vp, sz, i32, ctypes.c_double, vp, ctypes.POINTER(vp)]
        lib.fsm_serve_submit.argtypes = [vp, i64, i32, i32, ctypes.c_double, vp, vp]
        lib.fsm_serve_tick.argtypes = [vp, pi32]
        lib.fsm_serve_poll.argtypes = [vp, i32, pi64, i32, pi32, pi32]
        lib.fsm_serve_cancel.argtypes = [vp, i64]
        lib.fsm_serve_request_status.argtypes = [vp, i64, pi32, pi32]
        lib.fsm_serve_stats.argtypes = [vp, pi64, i32]
        lib.fsm_serve_destroy.argtypes = [vp]
        lib.fsm_serve_group_create.argtypes = [ctypes.POINTER(vp), i32, ctypes.c_double, ctypes.POINTER(vp)]
        lib.fsm_serve_group_tick.argtypes = [vp, pi32]
        lib.fsm_serve_group_poll.argtypes = [vp, i32, pi32]
        lib.fsm_serve_group_stats.argtypes = [vp, pi64, i32]
        lib.fsm_serve_group_destroy.argtypes = [vp]
        lib.fsm_last_error.argtypes = [ctypes.c_char_p, sz]
        for name in EXPORTS:
            getattr(lib, name).restype = ctypes.c_int
        _lib = lib
        return lib


def last_error() -> str:
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.fsm_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code: int) -> None:
    if code == FSM_OK:
        return
    msg = last_error()
    if code == FSM_ERR_UNSUPPORTED:
        raise UnsupportedProgram(code, msg)
    raise FsmError(code, msg)
