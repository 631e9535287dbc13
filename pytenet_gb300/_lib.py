"""
ctypes binding of libptn_gb300.so, the C ABI declared in include/pytenet_gb300.h.

The library is the only compute path of this package: if it is missing or was
built for another ABI, importing the engine raises instead of falling back to
any CPU code.
"""

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libptn_gb300.so")
ABI_VERSION = 3
KRYLOV_MAXITER = 64

PTN_OK, PTN_BAD_SHAPE, PTN_BREAKDOWN, PTN_NAN, PTN_TIMEOUT, PTN_CUDA_ERROR, PTN_UNSUPPORTED = range(7)
PREC_FP64, PREC_SPLIT_BF16 = 0, 1
TUNE_TC_SPLIT_WAVES, TUNE_ZGEMM_SPLIT_WAVES, TUNE_LARFB_TILE, TUNE_QR_CLUSTER = 0, 1, 2, 3
TUNE_KRYLOV_FUSED = 4
TUNE_QR_PANEL = 5
TUNE_TC_PERSISTENT = 6
TUNE_TC_SKIP_ZERO = 7


class PtnError(RuntimeError):
    """Raised when an entry point of the C ABI reports a failure."""

    def __init__(self, status, message):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class PtnShapeError(PtnError, AssertionError):
    """Shape / argument check failed (the reference raises AssertionError here)."""


_STATUS_NAMES = {PTN_OK: "PTN_OK", PTN_BAD_SHAPE: "PTN_BAD_SHAPE", PTN_BREAKDOWN: "PTN_BREAKDOWN",
                 PTN_NAN: "PTN_NAN", PTN_TIMEOUT: "PTN_TIMEOUT", PTN_CUDA_ERROR: "PTN_CUDA_ERROR",
                 PTN_UNSUPPORTED: "PTN_UNSUPPORTED"}


class c128(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def cval(z):
    z = complex(z)
    return c128(z.real, z.imag)


class DepthCtx(C.Structure):
    """Mirror of ptn_depth_ctx."""
    _fields_ = [("params", C.c_void_p), ("history", C.c_void_p), ("slot", C.c_int),
                ("site", C.c_int), ("nsites", C.c_int), ("kind", C.c_int), ("tol", C.c_double),
                ("log", C.c_void_p), ("log_count", C.c_void_p), ("log_capacity", C.c_int),
                ("check_from", C.c_int)]


DEPTH_RECORD = 64


class KrylovState(C.Structure):
    """Mirror of ptn_krylov_state."""
    _fields_ = [("m_used", C.c_int32), ("stopped", C.c_int32), ("maxiter", C.c_int32),
                ("status", C.c_int32), ("breakdowns", C.c_int32), ("m_target", C.c_int32),
                ("nrm", C.c_double), ("beta_next", C.c_double), ("eval0", C.c_double),
                ("resid", C.c_double), ("early_exits", C.c_int32), ("iters_total", C.c_int32),
                ("feat", C.c_float * 12), ("alpha", C.c_double * KRYLOV_MAXITER),
                ("beta", C.c_double * KRYLOV_MAXITER), ("coef", c128 * KRYLOV_MAXITER)]


P = C.c_void_p
I = C.c_int
L = C.c_long
S = C.c_size_t
D = C.c_double

# name -> (restype, argtypes)
_SIGS = {
    "ptn_abi_version": (I, []),
    "ptn_version": (C.c_char_p, []),
    "ptn_last_error": (C.c_char_p, []),
    "ptn_launch_count": (C.c_uint64, []),
    "ptn_tune_set": (I, [I, I]),
    "ptn_tune_get": (I, [I]),
    "ptn_prof_start": (None, [C.c_uint]),
    "ptn_prof_stop": (None, []),
    "ptn_prof_read": (I, [I, C.POINTER(D), C.POINTER(D), C.POINTER(D), C.POINTER(L)]),
    "ptn_heff_workspace_bytes": (S, [I, I, I, I, I, I]),
    "ptn_heff_apply": (I, [P, P, P, P, P, I, I, I, I, I, I, P, S, P]),
    "ptn_heff_noalloc_capacity_bytes": (S, []),
    "ptn_heff_apply_noalloc": (I, [P, P, P, P, P, I, I, I, I, I, P]),
    "ptn_bond_workspace_bytes": (S, [I, I, I, I]),
    "ptn_bond_apply": (I, [P, P, P, P, I, I, I, I, P, S, P]),
    "ptn_env_workspace_bytes": (S, [I, I, I, I, I, I]),
    "ptn_env_step_left": (I, [P, P, P, P, P, I, I, I, I, I, I, P, S, P]),
    "ptn_env_step_right": (I, [P, P, P, P, P, I, I, I, I, I, I, P, S, P]),
    "ptn_zgemm_workspace_bytes": (S, [I, I, I, I]),
    "ptn_zgemm": (I, [C.c_char, C.c_char, I, I, I, c128, P, L, L, P, L, L, c128, P, L, L, I, P, S,
                      P]),
    "ptn_zgemm_split_bf16_workspace_bytes": (S, [I, I, I]),
    "ptn_zgemm_split_bf16": (I, [P, L, P, L, P, L, I, I, I, P, S, P]),
    "ptn_tc_error": (I, []),
    "ptn_krylov_state_bytes": (S, []),
    "ptn_krylov_stop_flag": (P, [P]),
    "ptn_krylov_start": (I, [P, P, P, L, I, P]),
    "ptn_krylov_step": (I, [P, P, L, I, P]),
    "ptn_krylov_last": (I, [P, P, P, L, I, P]),
    "ptn_krylov_expm_coef": (I, [P, D, D, P]),
    "ptn_krylov_eigh_coef": (I, [P, P]),
    "ptn_krylov_combine": (I, [P, P, L, P, P]),
    "ptn_krylov_tridiag_eig": (I, [P, P, P, P]),
    "ptn_site_step_workspace_bytes": (S, [I, I, I, I, I, I]),
    "ptn_expm_site": (I, [P, P, P, P, I, I, I, I, I, D, D, I, I, P, P, P, S, P]),
    "ptn_bond_step_workspace_bytes": (S, [I, I, I, I]),
    "ptn_expm_bond": (I, [P, P, P, I, I, I, D, D, I, I, P, P, P, S, P]),
    "ptn_eigh_site": (I, [P, P, P, P, I, I, I, I, I, I, I, P, P, P, S, P]),
    "ptn_expm_site_ex": (I, [P, P, P, P, I, I, I, I, I, D, D, I, I, P, P, P, P, S, P]),
    "ptn_expm_bond_ex": (I, [P, P, P, I, I, I, D, D, I, I, P, P, P, P, S, P]),
    "ptn_depth_labels": (I, [P, I, I, D, P, P]),
    "ptn_mlp_param_count": (I, []),
    "ptn_mlp_workspace_bytes": (S, [I]),
    "ptn_mlp_forward": (I, [P, P, I, P, P]),
    "ptn_mlp_grad": (I, [P, P, P, I, P, P, P, S, P]),
    "ptn_mlp_adam": (I, [P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, I, P]),
    "ptn_svd_workspace_bytes": (S, [I, I]),
    "ptn_svd": (I, [P, I, I, L, P, L, P, P, L, P, P, S, P]),
    "ptn_diag_scale": (I, [P, L, L, L, P, I, P]),
    "ptn_qr_workspace_bytes": (S, [I, I]),
    "ptn_qr": (I, [P, I, I, P, L, P, L, P, S, P]),
    "ptn_gather": (I, [P, P, P, I, I, P, P]),
    "ptn_scatter": (I, [P, L, P, P, I, I, P, P]),
    "ptn_scale": (I, [P, P, L, c128, P]),
    "ptn_transpose_210": (I, [P, P, I, I, I, P]),
    "ptn_sign_fix": (I, [P, L, P, P, P]),
}

_lib = None
_lock = threading.Lock()


def load(path=None):
    """Load the shared library (once) and bind every declared entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or os.environ.get("PTN_GB300_LIB", LIB_PATH)
        if not os.path.exists(p):
            raise ImportError(
                f"pytenet_gb300: native library not found at {p}. Build it with "
                f"`python -c 'import __graft_entry__ as g; g.build()'` or "
                f"`python pytenet_gb300/build.py`. There is no CPU fallback.")
        lib = C.CDLL(p)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.ptn_abi_version() != ABI_VERSION:
            raise ImportError(f"pytenet_gb300: ABI mismatch ({lib.ptn_abi_version()} != {ABI_VERSION})")
        _lib = lib
        return lib


def exported_names():
    return list(_SIGS)


def check(status):
    """Turn a ptn_status into an exception."""
    if status == PTN_OK:
        return
    msg = _lib.ptn_last_error().decode(errors="replace") if _lib is not None else ""
    if status == PTN_BAD_SHAPE:
        raise PtnShapeError(status, msg)
    raise PtnError(status, msg)
