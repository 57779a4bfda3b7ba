"""ctypes binding of the C ABI in include/mpsim_gb300.h.

The library is the product's only compute path: if it (or a CUDA device) is
missing, every entry point raises -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmpsim_gb300.so")

MPS_OK = 0
MPS_ERR_ARG = 1
MPS_ERR_CUDA = 2
MPS_ERR_WORKSPACE = 3
MPS_ERR_NOT_CONVERGED = 4
MPS_ERR_NONFINITE = 5
MPS_ERR_TIMEOUT = 6
NOALLOC_SCRATCH_BYTES = 32 << 20       # MPS_NOALLOC_SCRATCH_BYTES

STATUS_NOT_CONVERGED = 1
STATUS_NONFINITE = 2
STATUS_TIMEOUT = 4
JOB_THETA_GIVEN = 1        # mps_2q_job.flags: a holds theta itself

# mps_2q_job, field for field (88 bytes).
JOB_DTYPE = np.dtype([
    ("a", np.uint64), ("b", np.uint64), ("gate", np.uint64),
    ("a_out", np.uint64), ("b_out", np.uint64), ("svals", np.uint64),
    ("discarded", np.uint64), ("status", np.uint64),
    ("chi_l", np.int32), ("chi_m", np.int32), ("chi_r", np.int32),
    ("k", np.int32), ("keep_left_canonical", np.int32), ("flags", np.int32),
])
assert JOB_DTYPE.itemsize == 88

# mps_1q_job (24 bytes).
JOB1_DTYPE = np.dtype([("site", np.uint64), ("gate", np.uint64),
                       ("chi_l", np.int32), ("chi_r", np.int32)])
assert JOB1_DTYPE.itemsize == 24


class SvdParams(ctypes.Structure):
    _fields_ = [("max_sweeps", ctypes.c_int32), ("tol", ctypes.c_float),
                ("block_cols", ctypes.c_int32), ("sweeps_out", ctypes.c_int32),
                ("wait_limit", ctypes.c_int32), ("stall_test", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("lq_off", ctypes.c_int32),
                ("block_request", ctypes.c_int32)]


PRECISION_PLAIN = 0       # MPS_PRECISION_PLAIN
PRECISION_MIXED = 1       # MPS_PRECISION_MIXED


# (name, restype, argtypes) for every symbol the header declares.
_P = ctypes.c_void_p
_I = ctypes.c_int
_SZ = ctypes.c_size_t
_LL = ctypes.c_longlong
SIGNATURES = {
    "mps_version": (_I, []),
    "mps_last_error": (ctypes.c_char_p, []),
    "mps_kernel_launches": (ctypes.c_ulonglong, []),
    "mps_apply_1q": (_I, [_P, _P, _I, _I, _I, _P]),
    "mps_apply_1q_batch": (_I, [_P, _P, _I, _I]),
    "mps_2q_workspace_bytes": (_SZ, [_I, _I, _I, _I]),
    "mps_2q_workspace_bytes_mixed": (_SZ, [_I, _I, _I, _I]),
    "mps_apply_2q_batch": (_I, [_P, _P, _I, _I, _I, _I, _P, _SZ, ctypes.POINTER(SvdParams)]),
    "mps_apply_2q_batch_noalloc": (_I, [_P, _P, _I, _I, _I, _I, ctypes.POINTER(SvdParams)]),
    "mps_sweep_workspace_bytes": (_SZ, [_I, _I]),
    "mps_inner_product": (_I, [_P, _P, _P, _P, _P, _I, _I, _P, _SZ, _P]),
    "mps_wavefunction": (_I, [_P, _P, _P, _I, _I, _P, _P, _SZ]),
    "mps_amplitudes": (_I, [_P, _P, _P, _I, _I, _P, _I, _P, _P, _SZ]),
    "mps_scale": (_I, [_P, _P, _SZ, ctypes.c_float, ctypes.c_float, _I]),
    "mps_cgemm": (_I, [_P, _I, _I, _I, _P, _LL, _LL, _I, _P, _LL, _LL, _I, _P, _LL, _LL, _I,
                       _LL, _LL, _LL]),
    "mps_cgemm_tc": (_I, [_P, _I, _I, _I, _P, _LL, _LL, _I, _P, _LL, _LL, _I, _P, _LL, _LL, _I,
                          _LL, _LL, _LL]),
    "mps_tc_error": (_I, [_P]),
    "mps_tc_profile": (_I, [_P, _I]),
    "mps_marginals_workspace_bytes": (_SZ, [_P, _I, _I]),
    "mps_site_marginals": (_I, [_P, _P, _P, _I, _I, _P, _SZ, _P]),
}

_lock = threading.Lock()
_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the shared library (once) and attach the C signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"mpsim_gb300: compiled library not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` "
                "(or python mpsim_gb300/build.py)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    msg = load().mps_last_error()
    return msg.decode() if msg else ""


class NativeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mpsim_gb300 native call failed ({code}): {msg}")
        self.code = code


def check(code: int) -> None:
    if code != MPS_OK:
        raise NativeError(code, last_error())
