"""ctypes binding of ``include/tn_mps.h`` (libtnmps.so).

Every entry point of the header is declared here with its argument types; the
loader fails loudly when the library is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import pathlib

from . import build as _build

u32, i32, u64, dbl = C.c_uint32, C.c_int32, C.c_uint64, C.c_double
P = C.POINTER
vp = C.c_void_p

TN_OK, TN_NONE, TN_CANCELLED = 0, 1, 2
STATUS = {
    0: "TN_OK", 1: "TN_NONE", 2: "TN_CANCELLED", -1: "TN_ERR_EMPTY_SYSTEM", -2: "TN_ERR_INVALID_QNUM",
    -3: "TN_ERR_UNPHYSICAL_INDEX", -4: "TN_ERR_STATE_SHAPE", -5: "TN_ERR_OPERATOR_SHAPE",
    -6: "TN_ERR_INVALID_ARG", -7: "TN_ERR_CUDA", -8: "TN_ERR_OOM", -9: "TN_ERR_CAPACITY",
    -10: "TN_ERR_NOT_CONVERGED", -11: "TN_ERR_PROB_SUM", -12: "TN_ERR_NO_DEVICE",
}
# device error-word bits (tn_*_device_status)
ST_NOT_CONVERGED, ST_CAPACITY, ST_PROB_SUM, ST_BAD_INSTR = 1, 2, 4, 8


class tn_trunc(C.Structure):
    _fields_ = [("mode", i32), ("chi_max", u32), ("cutoff", dbl)]


class tn_request(C.Structure):
    _fields_ = [("n", u32), ("trunc", tn_trunc), ("p", dbl), ("depth", u32), ("seed", u64), ("traj", u64)]


class tn_result(C.Structure):
    _fields_ = [("id", u64), ("layers", u32), ("final_entropy", dbl), ("latency_s", dbl), ("queue_s", dbl),
                ("status", i32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "tn_status_string": (C.c_char_p, [C.c_int]),
    "tn_last_error": (C.c_char_p, []),
    "tn_device_info": (C.c_int, [C.c_char_p, u32, P(u32)]),
    "tn_mps_new_qubits": (C.c_int, [u32, P(tn_trunc), i32, u32, P(vp)]),
    "tn_mps_free": (C.c_int, [vp]),
    "tn_mps_clone": (C.c_int, [vp, P(vp)]),
    "tn_mps_n": (C.c_int, [vp, P(u32)]),
    "tn_mps_precision": (C.c_int, [vp, P(i32)]),
    "tn_mps_get_trunc": (C.c_int, [vp, P(tn_trunc)]),
    "tn_mps_set_trunc": (C.c_int, [vp, P(tn_trunc)]),
    "tn_mps_from_vector": (C.c_int, [u32, P(dbl), u64, P(tn_trunc), i32, u32, P(vp)]),
    "tn_mps_import": (C.c_int, [u32, P(u32), P(dbl), P(dbl), P(tn_trunc), i32, u32, P(vp)]),
    "tn_mps_apply_unitary1": (C.c_int, [vp, u32, P(dbl), u32, u32]),
    "tn_mps_apply_unitary2": (C.c_int, [vp, u32, P(dbl), u32, u32]),
    "tn_mps_apply_unitary2_noalloc": (C.c_int, [vp, u32, P(dbl), u32, u32]),
    "tn_mps_probs": (C.c_int, [vp, u32, P(dbl)]),
    "tn_mps_prob": (C.c_int, [vp, u32, u32, P(dbl)]),
    "tn_mps_measure_prob": (C.c_int, [vp, u32, dbl, P(i32), P(dbl)]),
    "tn_mps_measure_postsel_prob": (C.c_int, [vp, u32, u32, P(dbl)]),
    "tn_mps_apply_meas_prob_layer": (C.c_int, [vp, P(u32), u32, P(i32), P(dbl), P(u32), P(i32), P(dbl), P(u32)]),
    "tn_mps_apply_bilayer": (C.c_int, [vp, P(u32), P(dbl), u32, P(u32), u32, P(dbl), P(u32), P(i32), P(dbl), P(u32)]),
    "tn_mps_entropy_vn": (C.c_int, [vp, u32, P(dbl)]),
    "tn_mps_entropy_ry_schmidt": (C.c_int, [vp, dbl, u32, P(dbl)]),
    "tn_mps_bond_dim": (C.c_int, [vp, u32, P(u32)]),
    "tn_mps_max_bond_dim": (C.c_int, [vp, P(u32)]),
    "tn_mps_svals": (C.c_int, [vp, u32, P(dbl), u32, P(u32)]),
    "tn_mps_export_gamma": (C.c_int, [vp, u32, P(dbl), u64, P(u32)]),
    "tn_mps_contract": (C.c_int, [vp, P(dbl), u64]),
    "tn_mps_device_status": (C.c_int, [vp, P(i32)]),
    "tn_mps_stats": (C.c_int, [vp, P(dbl), i32]),
    "tn_batch_create": (C.c_int, [u32, P(u32), P(tn_trunc), i32, P(u32), P(vp)]),
    "tn_batch_free": (C.c_int, [vp]),
    "tn_batch_reset": (C.c_int, [vp, u32, u32, P(tn_trunc)]),
    "tn_batch_import": (C.c_int, [vp, u32, u32, P(u32), P(dbl), P(dbl), P(tn_trunc)]),
    "tn_batch_export_gamma": (C.c_int, [vp, u32, u32, P(dbl), u64, P(u32)]),
    "tn_batch_step": (C.c_int, [vp, P(u32), u32, P(u32), P(u32), P(dbl), P(u32), P(u32), P(dbl),
                                P(i32), P(dbl), P(dbl)]),
    "tn_batch_step_post": (C.c_int, [vp, P(u32), u32, P(u32), P(u32), P(dbl), P(u32), P(u32), P(dbl),
                                     P(i32), P(i32), P(dbl), P(dbl)]),
    "tn_batch_device_inputs": (C.c_int, [vp, u32, u32] + [P(vp)] * 10),
    "tn_batch_step_device": (C.c_int, [vp, u32]),
    "tn_batch_step_ptrs": (C.c_int, [vp, u32] + [vp] * 11),
    "tn_batch_stats": (C.c_int, [vp, P(dbl), i32]),
    "tn_batch_synchronize": (C.c_int, [vp]),
    "tn_batch_bond_dims": (C.c_int, [vp, u32, P(u32), u32]),
    "tn_batch_svals": (C.c_int, [vp, u32, u32, P(dbl), u32, P(u32)]),
    "tn_batch_device_status": (C.c_int, [vp, P(i32)]),
    "tn_batch_slot_bytes": (C.c_int, [vp, u32, P(u64)]),
    "tn_batch_stream": (C.c_int, [vp, P(vp)]),
    "tn_batch_last_launch_ms": (C.c_int, [vp, P(C.c_float), P(C.c_float)]),
    "tn_batch_last_step_device_ms": (C.c_int, [vp, P(C.c_float)]),
    "tn_batch_set_queue_wait": (C.c_int, [vp, C.c_uint64, C.c_uint32]),
    "tn_batch_set_tuning": (C.c_int, [vp, i32, i32]),
    "tn_server_create": (C.c_int, [u64, u32, i32, u32, u32, P(vp)]),
    "tn_batch_set_schedule": (C.c_int, [vp, i32]),
    "tn_batch_autotune": (C.c_int, [vp, u32]),
    "tn_batch_set_theta_path": (C.c_int, [vp, i32]),
    "tn_batch_tuning": (C.c_int, [vp, P(i32), P(dbl)]),
    "tn_server_create_classes": (C.c_int, [u64, u32, i32, u32, u32, u32, u32, P(vp)]),
    "tn_server_class_stats": (C.c_int, [vp, u32, P(dbl)]),
    "tn_server_set_policy": (C.c_int, [vp, i32, u32, u32]),
    "tn_server_free": (C.c_int, [vp]),
    "tn_server_now": (C.c_int, [vp, P(dbl)]),
    "tn_server_submit": (C.c_int, [vp, P(tn_request), dbl, P(u64)]),
    "tn_server_tick": (C.c_int, [vp, P(u32), P(u32)]),
    "tn_server_poll": (C.c_int, [vp, P(tn_result), u32, P(u32)]),
    "tn_server_cancel": (C.c_int, [vp, u64]),
    "tn_server_history": (C.c_int, [vp, u64, P(dbl), u32, P(u32)]),
    "tn_server_stats": (C.c_int, [vp, P(dbl)]),
    "tn_haar_u4": (C.c_int, [P(dbl), P(dbl)]),
    "tn_gen_layer": (C.c_int, [u64, u64, u32, u32, dbl, P(u32), P(dbl), P(u32), P(u32), P(dbl), P(u32)]),
    "tn_gen_ginibre": (C.c_int, [u64, u64, u32, u32, P(dbl)]),
}

_LIB = None


class TnError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        detail = ""
        try:
            detail = lib().tn_last_error().decode()
        except Exception:  # pragma: no cover - best effort
            pass
        super().__init__(f"{what}: {STATUS.get(status, status)}" + (f" ({detail})" if detail else ""))


def library_path() -> pathlib.Path:
    return _build.SO


def lib() -> C.CDLL:
    """Load libtnmps.so (building it first if it is missing or stale)."""
    global _LIB
    if _LIB is None:
        so = _build.build()
        L = C.CDLL(str(so))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, what: str) -> int:
    if status < 0:
        raise TnError(status, what)
    return status


def dptr(a):
    return a.ctypes.data_as(P(dbl)) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(P(u32)) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(P(i32)) if a is not None else None
