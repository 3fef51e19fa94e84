"""ctypes binding of libva_gb300.so (the C ABI declared in include/va.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in this package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libva_gb300.so")

VA_OK = 0
STATUS_NAMES = {0: "VA_OK", 1: "VA_MAX_REJECTS", 2: "VA_MAX_STEPS", 3: "VA_NONFINITE",
                4: "VA_CKPT_BUDGET", 5: "VA_BAD_ARGS", 6: "VA_CUDA_ERROR", 7: "VA_NOT_READY",
                8: "VA_RECOMPUTE_MISMATCH", 9: "VA_NOT_RUN"}

MODELS = {"vdp": 0, "vdp_petsc": 1, "dho": 2, "glv": 3, "decay": 4, "glv_shared": 5, "user": 6}
TABLEAUX = {"dopri5": 0, "ck54": 1, "rkf78": 2, "rk4": 3, "euler": 4}
PRECISIONS = {"fp64": 0, "mixed": 1, "mixed_dw": 2}
COSTS = {"seeds": -1, "sumsq": 0, "sum": 1}

# Every symbol include/va.h declares (checked by the CPU test-suite).
EXPORTS = ["va_default_options", "va_create", "va_destroy", "va_forward", "va_backward",
           "va_gradient", "va_gradient_host", "va_forward_host", "va_backward_host", "va_gradient_noalloc",
           "va_autotune",
           "va_get_launch", "va_checkpoint_info",
           "va_trajectory", "va_set_adjoint_history", "va_adjoint_history", "va_adjoint_history_buffer",
           "va_set_shared", "va_last_error", "va_status_string", "va_probe_rate",
           "va_step_pow_undecided", "va_create_model", "va_forward_frozen", "va_contract_dA",
           "va_probe_mma_bf16", "va_matT_tc"]


class VaProblem(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("n", ctypes.c_int32), ("npar", ctypes.c_int32),
                ("batch", ctypes.c_int32), ("nout", ctypes.c_int32)]


class VaOptions(ctypes.Structure):
    _fields_ = [("tableau", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("atol", ctypes.c_double), ("rtol", ctypes.c_double), ("dt0", ctypes.c_double),
                ("max_steps", ctypes.c_int32), ("max_rejects", ctypes.c_int32),
                ("ckpt_budget_bytes", ctypes.c_int64), ("ckpt_stride", ctypes.c_int32),
                ("block_size", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("chunk_len", ctypes.c_int32), ("schedule", ctypes.c_int32),
                ("stage_records", ctypes.c_int32), ("step_pow", ctypes.c_int32),
                ("tensor_products", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2)]


class VaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load():
    """Loads the in-tree library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA library is required; there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, ip = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p
    H = ctypes.c_void_p
    L.va_default_options.argtypes = [ctypes.POINTER(VaOptions)]
    L.va_create.argtypes = [ctypes.POINTER(VaProblem), ctypes.POINTER(VaOptions), ctypes.POINTER(H)]
    L.va_destroy.argtypes = [H]
    L.va_forward.argtypes = [H, dp, dp, dp, dp, dp, ip, ip, ip, vp]
    L.va_backward.argtypes = [H, dp, dp, dp, dp, dp, ip, vp]
    L.va_gradient.argtypes = [H, ctypes.c_int32, dp, dp, dp, dp, dp, dp, dp, ip, ip, vp]
    L.va_gradient_host.argtypes = [H, ctypes.c_int32, dp, dp, dp, dp, dp, dp, dp, ip, ip, vp]
    L.va_forward_host.argtypes = [H, dp, dp, dp, dp, dp, ip, ip, ip]
    L.va_backward_host.argtypes = [H, dp, dp, dp, dp, dp, ip]
    i32, f64 = ctypes.c_int32, ctypes.c_double
    L.va_gradient_noalloc.argtypes = [i32, i32, i32, f64, f64, f64, i32, i32, i32, i32,
                                      dp, dp, dp, dp, dp, dp, dp, ip, ip, vp]
    L.va_autotune.argtypes = [H, ctypes.c_int32, dp, dp, dp, dp, vp]
    L.va_get_launch.argtypes = [H] + [ctypes.POINTER(ctypes.c_int32)] * 4
    L.va_checkpoint_info.argtypes = [H, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_int32)]
    L.va_trajectory.argtypes = [H, ctypes.c_int32, ctypes.c_int32, dp, dp, dp, ctypes.POINTER(ctypes.c_int32)]
    L.va_set_adjoint_history.argtypes = [H, ctypes.c_int32]
    L.va_adjoint_history.argtypes = [H, ctypes.c_int32, ctypes.c_int32, dp, dp, ctypes.POINTER(ctypes.c_int32)]
    L.va_adjoint_history_buffer.argtypes = [H, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int32)]
    L.va_set_shared.argtypes = [H, dp, dp]
    L.va_last_error.argtypes = [H]
    L.va_last_error.restype = ctypes.c_char_p
    L.va_status_string.argtypes = [ctypes.c_int32]
    L.va_status_string.restype = ctypes.c_char_p
    L.va_create_model.argtypes = [ctypes.POINTER(VaProblem), ctypes.POINTER(VaOptions), ctypes.c_void_p,
                                  ctypes.POINTER(H)]
    L.va_forward_frozen.argtypes = [H, ctypes.c_int32, ctypes.c_int32, dp, ip, dp, dp, dp, dp, vp]
    L.va_contract_dA.argtypes = [ctypes.c_int32, dp, dp, dp, vp]
    L.va_matT_tc.argtypes = [ctypes.c_int32, dp, dp, dp, vp]
    L.va_step_pow_undecided.argtypes = [H, ctypes.POINTER(ctypes.c_int64)]
    L.va_probe_rate.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double)]
    L.va_probe_mma_bf16.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    for name in EXPORTS:
        f = getattr(L, name)
        if f.restype is ctypes.c_int:  # default restype
            f.restype = ctypes.c_int32
    _lib = L
    return L
