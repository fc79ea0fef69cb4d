"""ctypes binding of ``libfockgb300.so`` (declared in ``include/fock_gb300.h``).

The library is the only compute path: if it is missing this module raises on
first use -- there is no CPU fallback.
"""

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libfockgb300.so")

FOCK_OK = 0
FOCK_ERR_INVALID = -1
FOCK_ERR_CUDA = -2
FOCK_ERR_UNSUPPORTED = -3

C64 = 0
C128 = 1

ROTATION = 1
KERR = 2
DISPLACEMENT = 3
SQUEEZE = 4
BEAMSPLITTER = 5
TWO_MODE_SQUEEZE = 6
MZGATE = 7
CROSS_KERR = 8
LOSS = 9
FOCK_BACKWARD_REUSE_BUILD = 1

TWO_MODE_KINDS = (BEAMSPLITTER, TWO_MODE_SQUEEZE, MZGATE, CROSS_KERR)
NPARAMS = {ROTATION: 1, KERR: 1, DISPLACEMENT: 2, SQUEEZE: 2, BEAMSPLITTER: 2, TWO_MODE_SQUEEZE: 2,
           MZGATE: 2, CROSS_KERR: 1, LOSS: 1}


class FockGate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("mode1", ctypes.c_int32), ("mode2", ctypes.c_int32),
                ("pidx", ctypes.c_int32)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("n_ops", ctypes.c_int32), ("n_gates", ctypes.c_int32), ("state_elems", ctypes.c_int64),
                ("state_bytes", ctypes.c_int64), ("workspace_bytes", ctypes.c_int64),
                ("flops_fwd", ctypes.c_int64), ("bytes_fwd", ctypes.c_int64), ("batch", ctypes.c_int32)]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_i64 = ctypes.c_int64
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

_SIGS = {
    "fock_last_error": (_i, [ctypes.c_char_p, ctypes.c_size_t]),
    "fock_version": (_i, []),
    "fock_gate_matrix_entries": (_i64, [_i, _i]),
    "fock_gate_workspace_bytes": (_i64, [_i, _i]),
    "fock_gate_matrix": (_i, [_i, _d, _d, _i, _vp, _vp, _vp, _vp]),
    "fock_expand_blocks": (_i, [_i, _i, _vp, _vp, _vp]),
    "fock_apply_gate": (_i, [_i, _d, _d, _i, _i, _i, _i, _i, _i, _dp, _vp, _vp, _vp, _vp, _vp]),
    "fock_apply_matrix1": (_i, [_vp, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "fock_gaussian_gate_matrix": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp]),
    "fock_apply_modes_workspace_bytes": (ctypes.c_int64, [_i, _i, _i]),
    "fock_apply_modes": (_i, [_i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fock_apply_phases": (_i, [_i, _i, _i, _i, _vp, _i, _ip, _dp, _vp, _vp, _vp]),
    "fock_mix": (_i, [_i, _i, _i, _vp, _vp, _vp]),
    "fock_vacuum": (_i, [_i, _i, _i, _i, _vp, _vp]),
    "fock_prepare_modes": (_i, [_i, _i, _i, _i, _ip, _vp, _vp, _vp, _vp, _vp]),
    "fock_prepare_workspace_bytes": (_i64, [_i, _i, _i, _i]),
    "fock_append_vacuum": (_i, [_i, _i, _i, _i, _i, _vp, _vp, _vp]),
    "fock_partial_trace": (_i, [_i, _i, _i, _i, _ip, _vp, _vp, _vp]),
    "fock_probs": (_i, [_i, _i, _i, _i, _vp, _vp, _vp]),
    "fock_marginals": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "fock_marginals_workspace_bytes": (_i64, [_i, _i, _i, _i]),
    "fock_reduced_dm1": (_i, [_i, _i, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "fock_reduced_dm1_workspace_bytes": (_i64, [_i, _i, _i, _i]),
    "fock_reduced_dm1_noalloc": (_i, [_i, _i, _i, _i, _i, _vp, _vp, _vp]),
    "fock_plan_create": (_i, [_i, _i, _i, _i, ctypes.POINTER(FockGate), _i, _i, ctypes.POINTER(_vp)]),
    "fock_plan_create_batch": (_i, [_i, _i, _i, _i, ctypes.POINTER(FockGate), _i, _i, _i, ctypes.POINTER(_vp)]),
    "fock_plan_destroy": (None, [_vp]),
    "fock_plan_get_info": (_i, [_vp, ctypes.POINTER(PlanInfo)]),
    "fock_plan_op": (_i, [_vp, _i, _ip, _ip, _ip, _ip]),
    "fock_plan_op_group": (_i, [_vp, _i, _ip, _ip, _ip]),
    "fock_plan_forward": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "fock_plan_backward": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fock_plan_backward_recompute": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _i, _vp, _vp]),
    "fock_plan_enable_timing": (_i, [_vp, _i]),
    "fock_plan_op_times": (_i, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "fock_plan_sweep_status": (_i, [_vp, _vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "fock_wigner": (_i, [_i, _vp, _vp, _i, _vp, _i, ctypes.c_double, _vp, _vp]),
    "fock_plan_tune": (_i, [_vp, _i, _i, _i, _i]),
    "fock_plan_op_config": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
}

_lock = threading.Lock()
_lib = None


def exported_symbols():
    """Names the header declares (used by the ABI tests)."""
    return sorted(_SIGS)


def load():
    """Load the library (once); raise ``RuntimeError`` if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIBPATH):
            raise RuntimeError(
                f"{LIBPATH} is missing: build the CUDA library first "
                "(python -m strawberryfields_gb300.build); there is no CPU fallback")
        lib = ctypes.CDLL(LIBPATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.fock_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, what=""):
    """Raise the Python exception matching a status code."""
    if rc == FOCK_OK:
        return
    msg = last_error()
    if what:
        msg = f"{what}: {msg}"
    if rc == FOCK_ERR_INVALID:
        raise ValueError(msg)
    if rc == FOCK_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    check(rc, name)
    return rc


def dptr(arr):
    """ctypes double* for a float64 numpy array (or None)."""
    if arr is None:
        return None
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    return arr.ctypes.data_as(_dp), arr
