"""ctypes binding of libitn_gpu.so (the C ABI in include/itn_gpu.h).

The library is required: when it is missing or cannot be loaded, every entry point
raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libitn_gpu.so")

ITN_OK, ITN_ERR_ARG, ITN_ERR_CUDA, ITN_ERR_OOM, ITN_ERR_NAN, ITN_ERR_TIMEOUT, \
    ITN_ERR_UNSUPPORTED, ITN_ERR_STATE = range(8)
F32, F64, C64, C128 = range(4)
SCHED_PARALLEL, SCHED_SEQUENTIAL = 0, 1
PREC_NATIVE, PREC_BF16, PREC_TF32, PREC_TF32X3 = 0, 1, 2, 3
MSG_IDENTITY_NORMALIZED, MSG_IDENTITY, MSG_ONES = 0, 1, 2
FAULT_WAIT_NS, FAULT_ALLOC, FAULT_STALL, FAULT_NO_PERSISTENT_ADJOINT, FAULT_NO_PERSISTENT_SWEEPS = 1, 2, 3, 4, 5

DTYPE_CODE = {np.dtype(np.float32): F32, np.dtype(np.float64): F64,
              np.dtype(np.complex64): C64, np.dtype(np.complex128): C128}
CODE_DTYPE = {v: k for k, v in DTYPE_CODE.items()}

#: every symbol the header declares (checked by the CPU tests)
EXPORTED = [
    "itn_abi_version", "itn_status_string", "itn_create", "itn_destroy", "itn_last_error",
    "itn_synchronize", "itn_graph_upload", "itn_graph_info", "itn_tensors_upload",
    "itn_tensors_upload_strided", "itn_tensors_download", "itn_messages_upload",
    "itn_messages_download", "itn_messages_init", "itn_bp_run", "itn_message_update",
    "itn_iterate_diff", "itn_logscalars", "itn_tc_selftest", "itn_bp_grad",
    "itn_sweep_vjp", "itn_logz_static_scratch", "itn_contraction_order", "itn_contract_network",
    "itn_apply_gates", "itn_bp_solve", "itn_bp_solve_submit", "itn_bp_solve_wait", "itn_inject_fault",
]


class GateDesc(ctypes.Structure):
    """itn_gate_desc (include/itn_gpu.h)."""
    _fields_ = [("nsite", ctypes.c_int32), ("d", ctypes.c_int32 * 2), ("nleg", ctypes.c_int32 * 2),
                ("bond", ctypes.c_int32), ("leg_dim", (ctypes.c_int32 * 6) * 2),
                ("site_off", ctypes.c_int64 * 2), ("env_off", (ctypes.c_int64 * 6) * 2),
                ("op_off", ctypes.c_int64), ("out_off", ctypes.c_int64 * 2), ("s_off", ctypes.c_int64)]


class ItnError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class ItnArgumentError(ItnError, ValueError):
    """Raised for ITN_ERR_ARG: the reference throws ArgumentError in these cases."""


class BpOpts(ctypes.Structure):
    _fields_ = [("schedule", ctypes.c_int32), ("maxiter", ctypes.c_int32),
                ("tol", ctypes.c_double), ("normalize", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("split_sweeps", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("edges", ctypes.c_void_p),
                ("n_edges", ctypes.c_int64)]


class GradOpts(ctypes.Structure):
    _fields_ = [("adjoint", ctypes.c_int32), ("maxiter", ctypes.c_int32), ("tol", ctypes.c_double),
                ("normalized", ctypes.c_int32), ("sweeps", ctypes.c_int32), ("checkpoint", ctypes.c_int32),
                ("reserved0", ctypes.c_int32)]


class GradResult(ctypes.Structure):
    _fields_ = [("adjoint_iterations", ctypes.c_int32), ("reserved0", ctypes.c_int32),
                ("adjoint_residual", ctypes.c_double), ("device_ms", ctypes.c_double)]


class BpResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("at_iteration", ctypes.c_int32),
                ("delta", ctypes.c_double), ("device_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int32), ("reserved0", ctypes.c_int32)]


_lock = threading.Lock()
_lib = None

_VP = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64


def _declare(lib):
    sig = {
        "itn_abi_version": (_I32, []),
        "itn_status_string": (ctypes.c_char_p, [_I32]),
        "itn_create": (_I32, [ctypes.POINTER(_VP), _I32, _I32]),
        "itn_destroy": (_I32, [_VP]),
        "itn_last_error": (ctypes.c_char_p, [_VP]),
        "itn_synchronize": (_I32, [_VP]),
        "itn_graph_upload": (_I32, [_VP, _I64, _VP, _VP, _VP, _VP, _VP, _I32, _VP]),
        "itn_graph_info": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
        "itn_tensors_upload": (_I32, [_VP, _I32, _VP]),
        "itn_tensors_upload_strided": (_I32, [_VP, _I32, _VP, _VP]),
        "itn_tensors_download": (_I32, [_VP, _I32, _VP]),
        "itn_messages_upload": (_I32, [_VP, _I32, _VP]),
        "itn_messages_download": (_I32, [_VP, _I32, _VP]),
        "itn_messages_init": (_I32, [_VP, _I32]),
        "itn_bp_run": (_I32, [_VP, ctypes.POINTER(BpOpts), ctypes.POINTER(BpResult)]),
        "itn_bp_solve": (_I32, [_VP, _I32, _VP, _VP, ctypes.POINTER(BpOpts), ctypes.POINTER(BpResult), _VP, _VP,
                                _VP]),
        "itn_bp_solve_submit": (_I32, [_VP, _I32, _VP, _VP, ctypes.POINTER(BpOpts), _VP, _I32]),
        "itn_bp_solve_wait": (_I32, [_VP, ctypes.POINTER(BpResult), _VP, _VP]),
        "itn_message_update": (_I32, [_VP, _I64, _I32]),
        "itn_iterate_diff": (_I32, [_VP, _I32, _VP, _VP, ctypes.POINTER(ctypes.c_double)]),
        "itn_logscalars": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
        "itn_tc_selftest": (_I32, [_VP, _VP, _VP, ctypes.POINTER(ctypes.c_double), _VP]),
        "itn_bp_grad": (_I32, [_VP, ctypes.POINTER(GradOpts), _VP, ctypes.POINTER(GradResult)]),
        "itn_sweep_vjp": (_I32, [_VP, _I32, _VP, _VP]),
        "itn_contraction_order": (_I32, [_I32, _VP, _VP, _VP, _I32, _VP]),
        "itn_contract_network": (_I32, [_VP, _I32, _I32, _VP, _VP, _VP, _VP, _I32, _VP, _I32, _VP, _I64,
                                        ctypes.POINTER(_I32), _VP, _VP, ctypes.POINTER(ctypes.c_double)]),
        "itn_logz_static_scratch": (_I32, [_I32, _VP, _I32, _I32, _I64, _I64, _I64, _VP, _VP, _VP, _VP,
                                           _VP, _VP, _VP, _VP, _VP, _VP, ctypes.c_char_p, _I32]),
        "itn_inject_fault": (_I32, [_VP, _I32, _I64]),
        "itn_apply_gates": (_I32, [_VP, _I32, _I64, _VP, _VP, _I64, _VP, _I64, _VP, _I64, _I32,
                                   ctypes.c_double, _I32, _VP, _I64, _VP, _I64, _VP,
                                   ctypes.POINTER(ctypes.c_double)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def load(path: str | None = None):
    """Load libitn_gpu.so (built by ``build.py``); raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise RuntimeError(
                    f"libitn_gpu.so not found at {p}: build it with "
                    "`python itensornetworksnext.jl_gb300/build.py` (no CPU fallback exists)")
            lib = ctypes.CDLL(p)
            _declare(lib)
            _lib = lib
    return _lib


def ptr(a):
    return None if a is None else a.ctypes.data


def check(ctx, status: int):
    if status == ITN_OK:
        return
    lib = load()
    msg = lib.itn_last_error(ctx).decode() if ctx else lib.itn_status_string(status).decode()
    if not msg:
        msg = lib.itn_status_string(status).decode()
    if status == ITN_ERR_ARG:
        raise ItnArgumentError(status, msg)
    raise ItnError(status, msg)
