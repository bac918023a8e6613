"""ctypes binding of libumwm_gb300.so (the C ABI declared in include/umwm_gpu.h).

The library is built in-tree by umwm_gb300/build.py.  There is no fallback:
if the shared library is missing, loading raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libumwm_gb300.so")

# every entry point of include/umwm_gpu.h
EXPORTS = [
    "umwm_gpu_put_gridtopo", "umwm_gpu_put_exclude", "umwm_gpu_put_forcing", "umwm_gpu_put_restart",
    "umwm_gpu_clear_inputs", "umwm_gpu_initialize", "umwm_gpu_initialize_text", "umwm_gpu_run",
    "umwm_gpu_finalize", "umwm_gpu_setup_host", "umwm_gpu_get_dims", "umwm_gpu_get_state", "umwm_gpu_set_state",
    "umwm_gpu_get_state_noalloc", "umwm_gpu_write_restart", "umwm_gpu_write_output",
    "umwm_gpu_get_field", "umwm_gpu_get_field_i", "umwm_gpu_get_screen", "umwm_gpu_set_option",
    "umwm_gpu_get_stat", "umwm_gpu_last_error", "umwm_gpu_ensemble_add", "umwm_gpu_ensemble_initialize",
    "umwm_gpu_select_member", "umwm_gpu_surrogate_init", "umwm_gpu_surrogate_get_params",
    "umwm_gpu_surrogate_set_params", "umwm_gpu_surrogate_capture", "umwm_gpu_surrogate_train",
    "umwm_gpu_surrogate_forward", "umwm_gpu_surrogate_grad", "umwm_gpu_surrogate_features", "umwm_gpu_surrogate_eval", "umwm_gpu_gemm_bf16",
]

ERRORS = {0: "UMWM_OK", 1: "UMWM_ERR_NAMELIST", 2: "UMWM_ERR_INPUT", 3: "UMWM_ERR_CUDA", 4: "UMWM_ERR_NONFINITE",
          5: "UMWM_ERR_TIMEOUT", 6: "UMWM_ERR_STATE", 7: "UMWM_ERR_ARG", 8: "UMWM_ERR_UNSUPPORTED"}


class UmwmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, str(code)), msg))
        self.code = code


_L = None


def lib():
    """Load the library once; raise if it has not been built."""
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(LIB_PATH):
        raise ImportError("libumwm_gb300.so is not built (%s); run python -c 'import __graft_entry__ as g; g.build()'"
                          % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    fp = ctypes.POINTER(ctypes.c_float)
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    c = ctypes.c_char_p
    sig = {
        "umwm_gpu_put_gridtopo": [c, fp, ctypes.c_int, ctypes.c_int],
        "umwm_gpu_put_exclude": [ip, ctypes.c_int],
        "umwm_gpu_put_forcing": [c, c, fp, ctypes.c_int, ctypes.c_int],
        "umwm_gpu_put_restart": [c, fp, ctypes.c_long, fp, ctypes.c_long],
        "umwm_gpu_clear_inputs": [],
        "umwm_gpu_initialize": [c],
        "umwm_gpu_initialize_text": [c],
        "umwm_gpu_run": [c, c],
        "umwm_gpu_finalize": [],
        "umwm_gpu_setup_host": [c],
        "umwm_gpu_get_dims": [ip],
        "umwm_gpu_get_state": [fp, fp],
        "umwm_gpu_set_state": [fp, fp],
        "umwm_gpu_get_state_noalloc": [fp, fp],
        "umwm_gpu_write_restart": [c],
        "umwm_gpu_write_output": [c],
        "umwm_gpu_get_field": [c, fp, ctypes.c_long],
        "umwm_gpu_get_field_i": [c, ip, ctypes.c_long],
        "umwm_gpu_get_screen": [dp, ctypes.c_long, ctypes.POINTER(ctypes.c_long)],
        "umwm_gpu_set_option": [c, ctypes.c_double],
        "umwm_gpu_ensemble_add": [c],
        "umwm_gpu_ensemble_initialize": [],
        "umwm_gpu_select_member": [ctypes.c_int],
        "umwm_gpu_surrogate_init": [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong],
        "umwm_gpu_surrogate_get_params": [fp, ctypes.c_long],
        "umwm_gpu_surrogate_set_params": [fp, ctypes.c_long],
        "umwm_gpu_surrogate_capture": [ctypes.c_long, ctypes.c_int],
        "umwm_gpu_surrogate_train": [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong, fp],
        "umwm_gpu_surrogate_forward": [fp, ctypes.c_int, fp],
        "umwm_gpu_surrogate_grad": [fp, fp, ctypes.c_int, fp, fp],
        "umwm_gpu_surrogate_features": [fp, ctypes.c_long],
        "umwm_gpu_surrogate_eval": [ctypes.c_long, ctypes.c_long, dp],
        "umwm_gpu_gemm_bf16": [ctypes.POINTER(ctypes.c_uint16), ctypes.POINTER(ctypes.c_uint16), fp, ctypes.c_int,
                               ctypes.c_int, ctypes.c_int],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.umwm_gpu_get_stat.argtypes = [c]
    L.umwm_gpu_get_stat.restype = ctypes.c_double
    L.umwm_gpu_last_error.argtypes = []
    L.umwm_gpu_last_error.restype = ctypes.c_char_p
    _L = L
    return L


def check(rc):
    if rc != 0:
        raise UmwmError(rc, lib().umwm_gpu_last_error().decode())
    return rc
