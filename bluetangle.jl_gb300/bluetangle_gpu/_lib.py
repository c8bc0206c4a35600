"""ctypes binding of libbtgpu.so (include/btgpu.h).

The library must exist: there is no CPU fallback.  Loading fails loudly when
the shared library has not been built (python bluetangle.jl_gb300/build.py)
and every call raises BTError with the library's message on a non-zero status.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("BTGPU_LIB", os.path.join(PKG, "libbtgpu.so"))

BT_OK = 0
BT_ERR_BAD_ARG = -1
BT_ERR_NOT_CPTP = -2
BT_ERR_OOM = -3
BT_ERR_DEVICE = -4
BT_ERR_TIMEOUT = -5
BT_ERR_UNSUPPORTED = -6
BT_ERR_NO_BRANCH = -7

BT_REPR_SV = 0
BT_REPR_DM = 1
BT_PREC_C128 = 0
BT_PREC_C64 = 1
BT_KRAUS_TRAJ = 0
BT_KRAUS_SUM = 1
BT_KRAUS_REF_ORDER = 0x100
BT_KRAUS_UNITARY_MIX = 0x200


class BTError(RuntimeError):
    """Error raised for a non-zero status of the engine (the reference throws a String)."""

    def __init__(self, code, msg):
        super().__init__(f"{msg} (status {code})")
        self.code = code


P = ctypes.c_void_p
i32, i64, u64, dbl = ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double

# name -> (restype, argtypes); the full exported surface of include/btgpu.h
SIGNATURES = {
    "bt_abi_version": (i32, []),
    "bt_status_string": (ctypes.c_char_p, [i32]),
    "bt_ctx_create": (i32, [i32, u64, ctypes.POINTER(P)]),
    "bt_ctx_destroy": (i32, [P]),
    "bt_last_error": (ctypes.c_char_p, [P]),
    "bt_ctx_synchronize": (i32, [P]),
    "bt_ctx_launch_count": (i32, [P, ctypes.POINTER(i64)]),
    "bt_ctx_stream": (i32, [P, ctypes.POINTER(P)]),
    "bt_state_alloc": (i32, [P, i32, i32, i32, i32, ctypes.POINTER(P)]),
    "bt_state_free": (i32, [P]),
    "bt_state_info": (i32, [P, P, P, P, P]),
    "bt_state_device_ptr": (P, [P]),
    "bt_state_set_zero": (i32, [P, i64]),
    "bt_state_set_basis": (i32, [P, i64, u64]),
    "bt_state_copy": (i32, [P, i64, P, i64]),
    "bt_state_upload": (i32, [P, i64, i64, i64, P]),
    "bt_state_download": (i32, [P, i64, i64, i64, P]),
    "bt_apply_matrix": (i32, [P, i32, P, P, i32, P, i64]),
    "bt_apply_kraus": (i32, [P, i32, P, i32, P, i32, P, P, P, P]),
    "bt_apply_matrix_members": (i32, [P, i32, P, P, i32, P]),
    "bt_measure_z": (i32, [P, i32, P, P, P, P]),
    "bt_measure_z2": (i32, [P, i32, i32, P, P, P, P]),
    "bt_reduced_dm": (i32, [P, i32, P, i64, P]),
    "bt_plan_create": (i32, [P, i32, i32, i32, ctypes.POINTER(P)]),
    "bt_plan_free": (i32, [P]),
    "bt_plan_add_matrix": (i32, [P, i32, P, P, i32, P]),
    "bt_plan_add_kraus_sum": (i32, [P, i32, P, i32, P]),
    "bt_plan_compile": (i32, [P, i32]),
    "bt_tc_tf32_peak": (i32, [P, i32, P]),
    "bt_plan_set_matrices": (i32, [P, i32, P, P]),
    "bt_plan_set_variable": (i32, [P, i32, P]),
    "bt_plan_stats": (i32, [P, P, P, P, P, P]),
    "bt_plan_cost": (i32, [P, P, P]),
    "bt_plan_pass_ops": (i32, [P, i64, P, P, P, P, i32, i32]),
    "bt_plan_run": (i32, [P, P, i64]),
    "bt_plan_run_members": (i32, [P, P, i32, P, P]),
    "bt_plan_prepare_members": (i32, [P, i32, P]),
    "bt_plan_member_table": (i32, [P, i64, i64, i32, P, P, P, i64, P]),
    "bt_plan_set_tuning": (i32, [P, i32, i32, i32, i32]),
    "bt_program_create": (i32, [P, i32, i32, i32, ctypes.POINTER(P)]),
    "bt_program_free": (i32, [P]),
    "bt_program_add_gate": (i32, [P, i32, P, P, i32]),
    "bt_program_add_channel": (i32, [P, i32, P, i32, P, i32, P]),
    "bt_program_add_measure": (i32, [P, i32, P]),
    "bt_program_set_range": (i32, [P, i64, i64]),
    "bt_program_prepare": (i32, [P, P]),
    "bt_program_info": (i32, [P, P, P, P]),
    "bt_program_set_gate": (i32, [P, i64, P]),
    "bt_program_run": (i32, [P, P, P, u64, P]),
    "bt_program_set_executor": (i32, [P, i32]),
    "bt_shadow_accumulate": (i32, [P, i64, P, P]),
    "bt_serve_create": (i32, [i32, i32, u64, u64, ctypes.POINTER(P)]),
    "bt_serve_destroy": (i32, [P]),
    "bt_serve_add_plan_client": (i32, [P, P, i32, P, P, P, P]),
    "bt_serve_add_program_client": (i32, [P, P, i32, P, P, P, P]),
    "bt_serve_add_packed_client": (i32, [P, P, i32, P, P, P, P]),
    "bt_serve_submit": (i32, [P, i64, i32, P, P, u64, P]),
    "bt_serve_poll": (i32, [P, i64, i64, P, P, P]),
    "bt_serve_stats": (i32, [P, P, P, P, P, P, P]),
    "bt_sample": (i32, [P, i64, i64, P, u64, P]),
    "bt_sample_members": (i32, [P, P, u64, P]),
    "bt_probabilities": (i32, [P, i64, P]),
    "bt_sample_noalloc": (i32, [P, i32, i32, i64, P, u64, u64, P, P]),
    "bt_expect_pauli": (i32, [P, i32, P, P, P, i64, P]),
    "bt_expect_z_all": (i32, [P, i64, P]),
    "bt_expect_matrix": (i32, [P, i32, P, P, i32, P, i64, P]),
    "bt_norm2": (i32, [P, i64, P]),
    "bt_fidelity": (i32, [P, i64, P, i64, P]),
    "bt_fidelity_dm": (i32, [P, i64, P, i64, P]),
    "bt_rho_accumulate": (i32, [P, i64, P, dbl]),
    "bt_state_random": (i32, [P, i64, u64]),
    "bt_state_clear": (i32, [P, i64]),
}

_lib = None


def lib():
    """Loads libbtgpu.so once; raises if it is missing (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libbtgpu.so not found at {LIB_PATH}: build it with "
                "`python bluetangle.jl_gb300/build.py` (CUDA toolkit required)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, ctx_ptr=None):
    if rc != BT_OK:
        msg = lib().bt_last_error(ctx_ptr)
        raise BTError(rc, msg.decode() if msg else lib().bt_status_string(rc).decode())
