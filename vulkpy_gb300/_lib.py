"""ctypes binding of ``libvulkpy_gb300.so`` (declarations in include/vulkpy_gb300.h).

This replaces the pybind11 module ``vulkpy._vkarray`` (vulkpy/_vkarray.cc:756-898).
The library must have been built (``vulkpy_gb300.build.build()``); importing
this module without it raises ImportError -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("VULKPY_GB300_LIB", _HERE / "libvulkpy_gb300.so"))

if not LIB_PATH.exists():
    raise ImportError(
        f"vulkpy_gb300 native library not found at {LIB_PATH}; "
        "build it with `python vulkpy_gb300/build.py` (needs nvcc)")

lib = C.CDLL(str(LIB_PATH))

# status codes
OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_TIMEOUT = 0, 1, 2, 3, 4

# op codes (enum vkc_binary_op / vkc_unary_op / vkc_reduce_op)
ADD, SUB, MUL, DIV, POW, MAX, MIN, RSUB, RDIV, RPOW = range(10)
UNARY = {name: i for i, name in enumerate(
    ["abs", "sign", "sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh", "tanh",
     "asinh", "acosh", "atanh", "exp", "log", "exp2", "log2", "sqrt", "invsqrt", "copy"])}
SUM, PROD, MAXIMUM, MINIMUM = range(4)
ARGMAX, ARGMIN = range(2)
RED_PLAIN, RED_PAIRWISE, RED_COMPENSATED = range(3)
MM_FP32, MM_BF16, MM_BF16X3 = range(3)
ACT_NONE, ACT_RELU, ACT_SIGMOID = range(3)
LOSS_CE, LOSS_SCE, LOSS_MSE, LOSS_HUBER = range(4)

vp = C.c_void_p
sz = C.c_size_t
i64 = C.c_int64
i32 = C.c_int
f32 = C.c_float
f64 = C.c_double
u32 = C.c_uint32
u64 = C.c_uint64
pi64 = C.POINTER(C.c_int64)
pvp = C.POINTER(C.c_void_p)


class GemmProblem(C.Structure):
    """struct vkc_gemm_problem (include/vulkpy_gb300.h)."""
    _fields_ = [("ta", C.c_int32), ("tb", C.c_int32), ("m", C.c_int64), ("n", C.c_int64), ("k", C.c_int64),
                ("alpha", C.c_float), ("beta", C.c_float), ("a", C.c_void_p), ("lda", C.c_int64),
                ("b", C.c_void_p), ("ldb", C.c_int64), ("c", C.c_void_p), ("ldc", C.c_int64),
                ("bias", C.c_void_p), ("act", C.c_int32), ("relu_mask", C.c_void_p)]


class GemmUpdate(C.Structure):
    """struct vkc_gemm_update (include/vulkpy_gb300.h)."""
    _fields_ = [("value", C.c_void_p), ("scale", C.c_float)]

_SIGS = {
    "vkc_last_error": ([], C.c_char_p),
    "vkc_version": ([], C.c_char_p),
    "vkc_device_count": ([C.POINTER(C.c_int)], i32),
    "vkc_device_open": ([i32, f32, C.POINTER(vp)], i32),
    "vkc_device_close": ([vp], i32),
    "vkc_device_synchronize": ([vp], i32),
    "vkc_device_stream": ([vp, C.POINTER(vp)], i32),
    "vkc_device_set_stream": ([vp, vp], i32),
    "vkc_device_info": ([vp, C.POINTER(C.c_int), C.c_char_p, sz], i32),
    "vkc_device_check_errors": ([vp, C.POINTER(u32)], i32),
    "vkc_alloc": ([vp, sz, C.POINTER(vp)], i32),
    "vkc_free": ([vp, vp], i32),
    "vkc_host_alloc": ([sz, C.POINTER(vp)], i32),
    "vkc_host_free": ([vp], i32),
    "vkc_upload": ([vp, vp, sz, C.POINTER(vp)], i32),
    "vkc_h2d": ([vp, vp, vp, sz, C.POINTER(vp)], i32),
    "vkc_upload_async": ([vp, vp, sz, C.POINTER(vp), C.POINTER(vp)], i32),
    "vkc_d2h_async": ([vp, vp, vp, sz, C.POINTER(vp)], i32),
    "vkc_stream_wait_job": ([vp, vp], i32),
    "vkc_d2h": ([vp, vp, vp, sz], i32),
    "vkc_fill_f32": ([vp, vp, sz, f32], i32),
    "vkc_fill_u32": ([vp, vp, sz, u32], i32),
    "vkc_copy": ([vp, vp, vp, sz], i32),
    "vkc_job_record": ([vp, C.POINTER(vp)], i32),
    "vkc_job_wait": ([vp, i64], i32),
    "vkc_job_query": ([vp, C.POINTER(C.c_int)], i32),
    "vkc_job_destroy": ([vp], i32),
    "vkc_timer_record": ([vp, C.POINTER(vp)], i32),
    "vkc_job_elapsed_ms": ([vp, vp, C.POINTER(C.c_float)], i32),
    "vkc_launch_count": ([C.POINTER(C.c_uint64)], i32),
    "vkc_alloc_count": ([C.POINTER(C.c_uint64)], i32),
    "vkc_set_pdl": ([i32], i32),
    "vkc_set_cluster_splitk": ([i32], i32),
    "vkc_side_defer": ([vp, i32], i32),
    "vkc_side_begin": ([vp], i32),
    "vkc_side_end": ([vp], i32),
    "vkc_inject_alloc_failure": ([i64], i32),
    "vkc_binary": ([vp, i32, vp, vp, vp, sz], i32),
    "vkc_binary_scalar": ([vp, i32, vp, f32, vp, sz], i32),
    "vkc_unary": ([vp, i32, vp, vp, sz], i32),
    "vkc_clamp": ([vp, vp, vp, vp, f32, f32, vp, sz], i32),
    "vkc_broadcast_binary": ([vp, i32, vp, pi64, vp, pi64, vp, pi64, i32], i32),
    "vkc_broadcast_clamp": ([vp, vp, pi64, vp, pi64, f32, vp, pi64, f32, vp, pi64, i32], i32),
    "vkc_broadcast_to": ([vp, vp, pi64, vp, pi64, i32], i32),
    "vkc_reduce_all": ([vp, i32, i32, vp, sz, vp, f32], i32),
    "vkc_reduce_axis": ([vp, i32, vp, sz, sz, sz, vp, i32, f32], i32),
    "vkc_reduce_all_noalloc": ([vp, i32, i32, vp, sz, vp, f32], i32),
    "vkc_matmul": ([vp, i32, vp, vp, vp, i64, i64, i64], i32),
    "vkc_gemm": ([vp, i32, i32, i32, i64, i64, i64, f32, vp, i64, vp, i64, f32, vp, i64], i32),
    "vkc_gemm_plan_set": ([i32, i64, i64, i64, i32, i32], i32),
    "vkc_gemm_plan_get": ([vp, i32, i64, i64, i64, C.POINTER(C.c_int), C.POINTER(C.c_int)], i32),
    "vkc_gemm_tune_set": ([i32, i64, i64, i64, i32], i32),
    "vkc_gemm_tune_get": ([vp, i32, i64, i64, i64, C.POINTER(C.c_int)], i32),
    "vkc_gemm_tune_clear": ([], i32),
    "vkc_gemm_grouped": ([vp, i32, C.POINTER(GemmProblem), i32], i32),
    "vkc_gemm_grouped_update": ([vp, i32, C.POINTER(GemmProblem), C.POINTER(GemmUpdate), i32], i32),
    "vkc_colsum_grouped": ([vp, pvp, pvp, pi64, pi64, i32, i32], i32),
    "vkc_colsum_update_grouped": ([vp, pvp, pvp, pi64, pi64, i32, i32, pvp, C.POINTER(f32)], i32),
    "vkc_sgd_update_grouped": ([vp, pvp, pvp, pi64, f64, i32], i32),
    "vkc_adam_update_grouped": ([vp, pvp, pvp, pvp, pvp, pvp, pi64, i32, f64, f64, f64, f64], i32),
    "vkc_fill_f32_grouped": ([vp, pvp, pi64, f32, i32], i32),
    "vkc_mse_grouped": ([vp, pvp, pvp, pvp, pi64, pi64, vp, i32], i32),
    "vkc_gather": ([vp, vp, sz, vp, sz, vp], i32),
    "vkc_set_gather_bins": ([i32], i32),
    "vkc_pool_reserved": ([vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], i32),
    "vkc_gather_axis": ([vp, vp, sz, sz, sz, vp, sz, vp], i32),
    "vkc_arg_reduce_all": ([vp, i32, vp, sz, vp], i32),
    "vkc_arg_reduce_axis": ([vp, i32, vp, sz, sz, sz, vp], i32),
    "vkc_xoshiro_permutation": ([vp, vp, u32, vp, sz], i32),
    "vkc_xoshiro_seed": ([vp, u64, u32, vp], i32),
    "vkc_xoshiro_u32": ([vp, vp, u32, vp, sz], i32),
    "vkc_xoshiro_f32": ([vp, vp, u32, vp, sz], i32),
    "vkc_xoshiro_normal": ([vp, vp, u32, vp, sz, f32, f32], i32),
    "vkc_box_muller": ([vp, vp, vp, sz, f32, f32], i32),
    "vkc_xoshiro_randrange": ([vp, vp, u32, vp, sz, u32, u32], i32),
    "vkc_dense_forward": ([vp, i32, vp, vp, vp, vp, i64, i64, i64, i32], i32),
    "vkc_dense_stack_forward": ([vp, i32, i32, vp, i64, pi64, pvp, pvp, C.POINTER(i32), pvp], i32),
    "vkc_dense_backward": ([vp, i32, vp, vp, vp, vp, vp, vp, i64, i64, i64], i32),
    "vkc_dense_backward_act": ([vp, i32, vp, vp, vp, vp, i32, vp, vp, vp, vp, i64, i64, i64], i32),
    "vkc_dense_backward_ex": ([vp, i32, vp, vp, vp, vp, i32, vp, vp, vp, vp, i64, i64, i64, i32], i32),
    "vkc_dense_backward_chain": ([vp, i32, vp, vp, vp, vp, i32, vp, vp, vp, i64, i64, i64, i32], i32),
    "vkc_softmax": ([vp, vp, vp, i64, i64], i32),
    "vkc_cross_entropy": ([vp, vp, vp, vp, vp, i64, i64, i32], i32),
    "vkc_adam_update": ([vp, vp, vp, vp, vp, sz, f64, f64, f64, f64, f64, f64], i32),
    "vkc_sgd_update": ([vp, vp, vp, sz, f64], i32),
    "vkc_adam_update_dev": ([vp, vp, vp, vp, vp, sz, f64, f64, f64, f64, vp], i32),
    "vkc_activation_backward": ([vp, i32, vp, vp, vp, sz], i32),
    "vkc_dense_forward_f64": ([vp, vp, vp, vp, vp, i64, i64, i64, i32], i32),
    "vkc_dense_backward_f64": ([vp, vp, vp, vp, vp, vp, vp, i64, i64, i64], i32),
    "vkc_activation_backward_f64": ([vp, i32, vp, vp, vp, sz], i32),
    "vkc_cross_entropy_f64": ([vp, vp, vp, vp, vp, i64, i64, i32], i32),
    "vkc_softmax_ce_backward_f64": ([vp, vp, vp, vp, sz, f64], i32),
    "vkc_softmax_ce_backward": ([vp, vp, vp, vp, sz, f32], i32),
    "vkc_softmax_ce_fused": ([vp, vp, vp, vp, vp, vp, i64, i64, f32, f32], i32),
    "vkc_jit_compile": ([vp, C.c_char_p, C.c_char_p, C.POINTER(vp)], i32),
    "vkc_jit_launch": ([vp, vp, C.POINTER(vp), i32, C.POINTER(vp), i32, sz], i32),
    "vkc_stream_create": ([vp, C.POINTER(vp)], i32),
    "vkc_stream_destroy": ([vp, vp], i32),
    "vkc_stream_wait": ([vp, vp, vp], i32),
    "vkc_graph_begin": ([vp], i32),
    "vkc_graph_end": ([vp, C.POINTER(vp)], i32),
    "vkc_graph_launch": ([vp], i32),
    "vkc_graph_destroy": ([vp], i32),
    "vkc_adagrad_update": ([vp, vp, vp, vp, sz, f64, f64], i32),
    "vkc_loss_rows": ([vp, i32, vp, vp, vp, vp, i64, i64], i32),
    "vkc_loss_rows_f64": ([vp, i32, vp, vp, vp, vp, i64, i64], i32),
    "vkc_loss_backward": ([vp, i32, C.POINTER(C.c_int), C.POINTER(f64), C.POINTER(f64), i32, vp, vp, vp, vp, sz],
                          i32),
    "vkc_loss_backward_f64": ([vp, i32, C.POINTER(C.c_int), C.POINTER(f64), C.POINTER(f64), i32, vp, vp, vp, vp,
                               sz], i32),
    "vkc_softmax_backward": ([vp, vp, vp, vp, i64, i64], i32),
    "vkc_softmax_backward_f64": ([vp, vp, vp, vp, i64, i64], i32),
    "vkc_activation_forward": ([vp, i32, vp, vp, sz], i32),
    "vkc_activation_forward_f64": ([vp, i32, vp, vp, sz], i32),
    "vkc_softmax_f64": ([vp, vp, vp, i64, i64], i32),
}

for _name, (_args, _res) in _SIGS.items():
    _fn = getattr(lib, _name)
    _fn.argtypes = _args
    _fn.restype = _res


class TimeoutError_(RuntimeError):
    """Raised when a wait deadline passes ("Timeout at Command Wait")."""


def last_error() -> str:
    return lib.vkc_last_error().decode(errors="replace")


def check(status: int) -> None:
    """Raise on a non-zero status, with the library's message."""
    if status == OK:
        return
    msg = last_error()
    if status == ERR_INVALID:
        raise ValueError(msg)
    if status == ERR_OOM:
        raise MemoryError(msg)
    if status == ERR_TIMEOUT:
        raise TimeoutError_(msg)
    raise RuntimeError(msg)


def shape_arg(shape) -> "C.Array":
    return (C.c_int64 * max(1, len(shape)))(*[int(s) for s in shape])


def exported_symbols() -> list[str]:
    return sorted(_SIGS)
