"""ctypes binding of libestl_cuda.so (include/estl_cuda.h).

The shared library is the product: it is loaded from the package directory
and a missing library is an error, never a reason to fall back to another
implementation.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libestl_cuda.so")

STATUS = {
    0: "ESTL_OK",
    1: "ESTL_INVALID_ARG",
    2: "ESTL_UNSUPPORTED_SIZE",
    3: "ESTL_OUT_OF_MEMORY",
    4: "ESTL_ADMISSION_REJECTED",
    5: "ESTL_DEVICE_ERROR",
    6: "ESTL_TIMEOUT",
    7: "ESTL_NOT_INITIALIZED",
}

FORWARD = -1
BACKWARD = +1
LAYOUT_INTERLEAVED = 0
LAYOUT_BLOCK_PLANAR = 1  # 32 real parts then 32 imaginary parts per block (PlannarizedDataInterface)
LAYOUT_SPLIT = 2         # all real parts, then all imaginary parts
PREC_FP32 = 0
PREC_SPLIT_FP16 = 1    # fp16 hi+lo tensor-core radix-16 stages (butterflies scaled by powers of two)
PREC_SPLIT_BF16 = 2    # bf16 hi+lo
PREC_SPLIT_BF16X3 = 3  # bf16 hi+mid+lo


class EstlError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.name = STATUS.get(status, str(status))


_lib = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_SZ = ctypes.c_size_t
_INT = ctypes.c_int

# name -> (restype, argtypes); the C declarations are in include/estl_cuda.h
SIGNATURES = {
    "estl_init": (_INT, [_INT, _SZ]),
    "estl_shutdown": (_INT, []),
    "estl_last_error": (ctypes.c_char_p, []),
    "estl_status_string": (ctypes.c_char_p, [_INT]),
    "estl_max_batch": (_I64, [_I64]),
    "estl_plan_create": (_INT, [_I64, _I64, _INT, _INT, ctypes.POINTER(_P)]),
    "estl_plan_create_ex": (_INT, [_I64, _I64, _INT, _INT, _P, ctypes.POINTER(_P)]),
    "estl_plan2d_create": (_INT, [_I64, _I64, _I64, _INT, _INT, ctypes.POINTER(_P)]),
    "estl_layout_floats": (_I64, [_INT, _I64]),
    "estl_execute_layout": (_INT, [_P, _INT, _P, _P, _P]),
    "estl_execute_host_layout": (_INT, [_P, _INT, _P, _P]),
    "estl_plan_destroy": (_INT, [_P]),
    "estl_plan_describe": (_INT, [_P, ctypes.c_char_p, _SZ]),
    "estl_plan_launches": (_I64, [_P]),
    "estl_plan_check": (_INT, [_P]),
    "estl_execute": (_INT, [_P, _P, _P, _P]),
    "estl_execute_host": (_INT, [_P, _P, _P]),
    "estl_plan_set_profiling": (_INT, [_P, _INT]),
    "estl_plan_kernel_stats": (_INT, [_P, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double)]),
    "estl_host_register": (_INT, [_P, _SZ]),
    "estl_host_unregister": (_INT, [_P]),
    "estl_autotune": (_INT, [_I64, _I64, _INT, ctypes.c_char_p, _SZ]),
    "estl_memory_usage": (_INT, [ctypes.POINTER(_SZ), ctypes.POINTER(_SZ)]),
    "estl_execute_noalloc": (_INT, [_I64, _I64, _INT, _P, _P, _P]),
    "estl_conv_output_length": (_I64, [_I64, _I64, _INT]),
    "estl_conv_workspace_size": (_INT, [_P, _I64, _INT, ctypes.POINTER(_SZ)]),
    "estl_conv_execute": (_INT, [_P, _I64, _INT, _P, _P, _P, _P, _SZ, _P]),
    "estl_conv_plan_create": (_INT, [_I64, _I64, _I64, _INT, ctypes.POINTER(_P)]),
    "estl_conv_plan_set_filter": (_INT, [_P, _P, _P]),
    "estl_conv_plan_execute": (_INT, [_P, _P, _P, _P]),
    "estl_conv_plan_launches": (_I64, [_P]),
    "estl_conv_plan_destroy": (_INT, [_P]),
    "estl_conv2d_output_size": (_INT, [_I64, _I64, _I64, _I64, _INT, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "estl_conv2d_plan_create": (_INT, [_I64, _I64, _I64, _I64, _I64, _INT, ctypes.POINTER(_P)]),
    "estl_conv2d_plan_set_filter": (_INT, [_P, _P, _P]),
    "estl_conv2d_plan_execute": (_INT, [_P, _P, _P, _P]),
    "estl_conv2d_plan_launches": (_I64, [_P]),
    "estl_conv2d_plan_destroy": (_INT, [_P]),
    "estl_conv2d_host": (_INT, [_I64, _I64, _I64, _I64, _INT, _P, _P, _P]),
    "estl_packed_plan_create": (_INT, [_P, _P, _I64, _INT, _INT, ctypes.POINTER(_P)]),
    "estl_packed_execute": (_INT, [_P, _P, _P, _P]),
    "estl_packed_check": (_INT, [_P]),
    "estl_packed_plan_set_test_hook": (_INT, [_P, _INT, ctypes.c_uint64]),
    "estl_packed_plan_describe": (_INT, [_P, ctypes.c_char_p, _SZ]),
    "estl_packed_plan_destroy": (_INT, [_P]),
    "estl_execute_packed": (_INT, [_P, _P, _I64, _INT, _P, _P, _P]),
    "estl_packed_mixed_plan_create": (_INT, [_P, _P, _I64, _INT, _P, _I64, _INT, _INT, ctypes.POINTER(_P)]),
    "estl_packed_mixed_execute": (_INT, [_P, _P, _P, _P, _P, _P, _P]),
    "estl_serve_start": (_INT, [_P, ctypes.POINTER(_P)]),
    "estl_serve_submit": (_INT, [_P, _P, ctypes.POINTER(ctypes.c_uint64)]),
    "estl_serve_poll": (_INT, [_P, ctypes.c_uint64, _INT, _P]),
    "estl_serve_stats_get": (_INT, [_P, _P]),
    "estl_serve_stop": (_INT, [_P]),
}


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_inflight_batches", ctypes.c_int),
                ("max_batch_requests", ctypes.c_int), ("max_queue", ctypes.c_int64)]


class ServeRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("direction", ctypes.c_int), ("flags", ctypes.c_int), ("reserved", ctypes.c_int),
                ("n", ctypes.c_int64), ("signal_len", ctypes.c_int64), ("filter_len", ctypes.c_int64),
                ("in_", ctypes.c_void_p), ("filter", ctypes.c_void_p), ("out", ctypes.c_void_p)]


class ServeResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("batch_requests", ctypes.c_int), ("latency_us", ctypes.c_double),
                ("queue_us", ctypes.c_double), ("device_us", ctypes.c_double)]


class ServeStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("rejected", ctypes.c_int64),
                ("batches", ctypes.c_int64), ("max_batch_requests", ctypes.c_int64), ("queued", ctypes.c_int64),
                ("inflight_bytes", ctypes.c_uint64), ("max_inflight_bytes", ctypes.c_uint64)]


REQ_FFT = 0
REQ_CONV = 1


class PlanOptions(ctypes.Structure):
    """estl_plan_options: mode 0 auto, 1 single tile (or cluster tile), 2 four-step,
    4 three-pass; explicit_tiles != 0 fixes the tile kernels (-1 fields: planner's choice)."""
    _fields_ = [("mode", ctypes.c_int), ("lag", ctypes.c_int), ("chunk", ctypes.c_int64),
                ("explicit_tiles", ctypes.c_int), ("split_log2", ctypes.c_int),
                ("single_loge", ctypes.c_int), ("single_logc", ctypes.c_int),
                ("col_loge", ctypes.c_int), ("col_logc", ctypes.c_int),
                ("row_loge", ctypes.c_int), ("row_logc", ctypes.c_int), ("pipelined", ctypes.c_int),
                ("split2_log2", ctypes.c_int), ("single_logr", ctypes.c_int), ("col_logr", ctypes.c_int),
                ("row_logr", ctypes.c_int), ("single_cluster_log2", ctypes.c_int)]


class ConvRequest(ctypes.Structure):
    """estl_conv_request: lengths and float offsets of one convolution."""
    _fields_ = [("signal_len", ctypes.c_int64), ("filter_len", ctypes.c_int64), ("signal_offset", ctypes.c_int64),
                ("filter_offset", ctypes.c_int64), ("output_offset", ctypes.c_int64)]


CONV_CORRELATE = 1
CONV_REFERENCE_COMPAT = 2


def conv_precision(p):
    """ESTL_CONV_PRECISION: the split precision of a convolution's FFT stages, or'd into its flags."""
    return int(p) << 8


def lib():
    """Load libestl_cuda.so (built by estl_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(the FFT engine has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    """Raise EstlError for a non-zero estl_status."""
    if status != 0:
        msg = lib().estl_last_error()
        raise EstlError(status, msg.decode() if msg else "")
    return status
