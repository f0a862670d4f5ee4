"""ctypes binding of the engine's C ABI (``include/pyramaterised_gb300.h``).

The library is loaded from ``pyramaterised_gb300/lib/libpqc_gb300.so``.  There
is no fallback: if the library is missing, or no CUDA device is present,
every engine call raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

PQC_OP_RX, PQC_OP_RY, PQC_OP_RZ, PQC_OP_MAT1, PQC_OP_CNOT, PQC_OP_CZ = 1, 2, 3, 4, 5, 6
PQC_OP_RXX, PQC_OP_RYY, PQC_OP_RZZ, PQC_OP_MAT2, PQC_OP_FSIM, PQC_OP_FIXED_FSIM = 7, 8, 9, 10, 11, 12
PQC_OP_PAULI, PQC_OP_FSIM_DTHETA, PQC_OP_FSIM_DPHI, PQC_OP_FIXED_FSIM_DTHETA = 13, 14, 15, 16
PQC_STATUS_LOAD_TIMEOUT = 1
PAULI_LETTER = {"I": 0, "X": 1, "Y": 2, "Z": 3}

# numpy mirror of `pqc_op` (320 bytes) and `pqc_pauli_term` (32 bytes)
OP_DTYPE = np.dtype(
    [
        ("kind", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("param", "<i4"), ("param2", "<i4"),
        ("sel", "<i4"), ("pauli", "<i4"), ("pad", "<i4"),
        ("scale", "<f8"), ("offset", "<f8"), ("scale2", "<f8"), ("offset2", "<f8"),
        ("m", "<f8", (32,)),
    ]
)
TERM_DTYPE = np.dtype([("xmask", "<u8"), ("zmask", "<u8"), ("coef", "<f8"), ("n_y", "<i4"), ("pad", "<i4")])
# numpy mirror of `pqc_run_item` (64 bytes): device and program pointers as uint64
RUN_ITEM_DTYPE = np.dtype([("prog", "<u8"), ("theta", "<u8"), ("theta_stride", "<i8"), ("batch", "<i8"),
                           ("psi0", "<u8"), ("psi0_index", "<i8"), ("row_limit", "<u8"), ("psi", "<u8")])
assert OP_DTYPE.itemsize == 320 and TERM_DTYPE.itemsize == 32 and RUN_ITEM_DTYPE.itemsize == 64

EXPORTS = [
    "pqc_abi_version", "pqc_last_error", "pqc_launch_count", "pqc_plan_order", "pqc_derivative_plan_order",
    "pqc_program_create", "pqc_program_destroy", "pqc_program_info",
    "pqc_program_set_occupancy", "pqc_program_set_launch", "pqc_program_limit_ok", "pqc_program_status",
    "pqc_run_workspace_size", "pqc_run", "pqc_run_limited", "pqc_run_fp64", "pqc_run_c64", "pqc_run_plain", "pqc_run_static_capacity", "pqc_run_static",
    "pqc_run_multi_workspace_size", "pqc_run_multi",
    "pqc_overlaps_workspace_size", "pqc_overlaps", "pqc_fidelity_hist_workspace_size", "pqc_fidelity_hist",
    "pqc_histogram", "pqc_expr_kl", "pqc_mw_workspace_size", "pqc_mw", "pqc_expect_workspace_size", "pqc_expect",
    "pqc_magic_workspace_size", "pqc_magic", "pqc_qfim_workspace_size", "pqc_qfim", "pqc_qfim_fp64", "pqc_gram_tf32_workspace_size", "pqc_gram_tf32",
    "pqc_gram_cross_workspace_size", "pqc_gram_cross",
    "pqc_derivative_states_workspace_size", "pqc_derivative_states", "pqc_derivative_states_from",
    "pqc_energy_grad_workspace_size", "pqc_energy_grad", "pqc_energy_grad_plain",
    "pqc_derivative_states_plain_workspace_size", "pqc_derivative_states_plain",
]

_lib = None

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
f64 = C.c_double
sz = C.c_size_t


class EngineError(RuntimeError):
    pass


def _sig(lib):
    S = {
        "pqc_abi_version": (i32, []),
        "pqc_last_error": (C.c_char_p, []),
        "pqc_launch_count": (C.c_longlong, []),
        "pqc_plan_order": (i32, [vp, i32, i32, i32, vp, vp, C.POINTER(i32)]),
        "pqc_derivative_plan_order": (i32, [vp, i32, vp, vp, i32, i32, i32, vp, C.POINTER(i32)]),
        "pqc_program_create": (i32, [vp, i32, i32, i32, i32, C.POINTER(vp)]),
        "pqc_program_destroy": (None, [vp]),
        "pqc_program_info": (i32, [vp, C.POINTER(i32), C.POINTER(i32)]),
        "pqc_program_set_occupancy": (i32, [vp, i32]),
        "pqc_program_set_launch": (i32, [vp, i32, i32]),
        "pqc_program_limit_ok": (i32, [vp, i32]),
        "pqc_program_status": (i32, [vp, C.POINTER(C.c_int32)]),
        "pqc_run_workspace_size": (sz, [vp, i64]),
        "pqc_run": (i32, [vp, vp, i64, i64, vp, i64, vp, vp, sz, vp]),
        "pqc_run_limited": (i32, [vp, vp, i64, i64, vp, i64, vp, vp, vp, sz, vp]),
        "pqc_run_fp64": (i32, [vp, vp, i64, i64, vp, i64, vp, vp, sz, vp]),
        "pqc_run_c64": (i32, [vp, vp, i64, i64, vp, i64, vp, vp, sz, vp]),
        "pqc_run_plain": (i32, [vp, vp, i64, i64, vp, i64, vp, vp, sz, vp]),
        "pqc_run_static_capacity": (sz, []),
        "pqc_run_static": (i32, [vp, vp, i64, i64, vp, i64, vp, vp]),
        "pqc_run_multi_workspace_size": (sz, [vp, i32]),
        "pqc_run_multi": (i32, [vp, i32, vp, sz, vp]),
        "pqc_overlaps_workspace_size": (sz, [i64, i32]),
        "pqc_overlaps": (i32, [vp, vp, vp, vp, i64, i32, vp, vp, sz, vp]),
        "pqc_fidelity_hist_workspace_size": (sz, [i64, i32]),
        "pqc_fidelity_hist": (i32, [vp, i64, i32, i32, vp, vp, vp, vp, sz, vp]),
        "pqc_histogram": (i32, [vp, i64, i32, vp, vp, vp]),
        "pqc_expr_kl": (i32, [vp, i32, vp, f64, vp, vp]),
        "pqc_mw_workspace_size": (sz, [i64, i32]),
        "pqc_mw": (i32, [vp, i64, i32, vp, vp, sz, vp]),
        "pqc_expect_workspace_size": (sz, [i64, i32, i32]),
        "pqc_expect": (i32, [vp, i64, i32, vp, i32, vp, vp, sz, vp]),
        "pqc_magic_workspace_size": (sz, [i64, i32]),
        "pqc_magic": (i32, [vp, i64, i32, f64, vp, vp, sz, vp]),
        "pqc_qfim_workspace_size": (sz, [i64, i32]),
        "pqc_qfim": (i32, [vp, vp, i64, i32, vp, vp, sz, vp]),
        "pqc_qfim_fp64": (i32, [vp, vp, i64, i32, vp, vp, sz, vp]),
        "pqc_gram_tf32_workspace_size": (sz, [i64, i32]),
        "pqc_gram_tf32": (i32, [vp, i64, i32, vp, vp, vp, sz, vp]),
        "pqc_gram_cross_workspace_size": (sz, [i64, i64, i32]),
        "pqc_gram_cross": (i32, [vp, i64, vp, i64, i32, vp, vp, sz, vp]),
        "pqc_derivative_states_workspace_size": (sz, [vp, i32, i32]),
        "pqc_derivative_states": (i32, [vp, vp, vp, i64, vp, vp, i32, i32, vp, vp, vp, sz, vp]),
        "pqc_derivative_states_from": (i32, [vp, vp, vp, vp, vp, vp, vp, i32, i32, vp, vp, sz, vp]),
        "pqc_energy_grad_workspace_size": (sz, [vp, i64, i32, i32]),
        "pqc_energy_grad": (i32, [vp, vp, i64, i64, vp, i64, vp, i32, vp, vp, i32, i32, vp, vp, vp, vp, sz, vp]),
        "pqc_energy_grad_plain": (i32, [vp, vp, i64, i64, vp, i64, vp, i32, vp, vp, i32, i32, vp, vp, vp, sz, vp]),
        "pqc_derivative_states_plain_workspace_size": (sz, [vp, i32]),
        "pqc_derivative_states_plain": (i32, [vp, vp, vp, i64, vp, vp, i32, vp, vp, sz, vp]),
    }
    for name, (res, args) in S.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def load(path=None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.lib_path()
    if not os.path.exists(path):
        raise EngineError(
            f"pyramaterised_gb300 CUDA library not found at {path}; build it with "
            "`python -m pyramaterised_gb300.build` (there is no CPU fallback)"
        )
    lib = C.CDLL(path)
    _sig(lib)
    if lib.pqc_abi_version() != 2:
        raise EngineError("ABI version mismatch")
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = _lib.pqc_last_error().decode(errors="replace") if _lib is not None else "?"
        raise EngineError(f"engine call failed ({rc}): {msg}")


def last_error():
    return load().pqc_last_error().decode(errors="replace")
