"""The C-ABI library loads and exports every symbol include/vulkpy_gb300.h declares
(no compute calls: runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vulkpy_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vkc_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert len(syms) >= 45
    assert "vkc_binary" in syms and "vkc_xoshiro_seed" in syms


def test_library_exports_every_declared_symbol():
    from vulkpy_gb300 import _lib
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_covers_header():
    from vulkpy_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.exported_symbols())


def test_version_and_error_strings():
    from vulkpy_gb300 import _lib
    assert b"sm_103a" in _lib.lib.vkc_version()
    assert isinstance(_lib.last_error(), str)


def test_null_device_is_rejected_without_gpu():
    from vulkpy_gb300 import _lib
    st = _lib.lib.vkc_binary(None, _lib.ADD, None, None, None, 4)
    assert st == _lib.ERR_INVALID
    assert "NULL" in _lib.last_error()


def test_gemm_tuning_table_host_side(tmp_path):
    """The split-K table is host state: set/clear validate without a GPU, and a
    table file round-trips through the loader."""
    import json
    from vulkpy_gb300 import _lib, autotune
    assert _lib.lib.vkc_gemm_tune_set(_lib.MM_BF16X3, 256, 1024, 784, 65) == _lib.ERR_INVALID
    assert _lib.lib.vkc_gemm_tune_set(_lib.MM_BF16X3, 256, 1024, 784, 4) == _lib.OK
    assert _lib.lib.vkc_gemm_tune_set(_lib.MM_BF16X3, 256, 1024, 784, 0) == _lib.OK   # erase
    assert _lib.lib.vkc_gemm_plan_set(_lib.MM_BF16, 256, 1024, 784, 4, 96) == _lib.ERR_INVALID
    assert _lib.lib.vkc_gemm_plan_set(_lib.MM_BF16, 256, 1024, 784, 4, 128) == _lib.OK
    assert _lib.lib.vkc_gemm_plan_set(_lib.MM_BF16, 256, 1024, 784, 0, 128) == _lib.OK   # erase
    p = tmp_path / "t.json"
    p.write_text(json.dumps({"bf16x3": [[8, 10, 10, 2], [7, 12, 14, 8, 128]], "bf16": [[8, 10, 10, 3, 256]]}))
    assert autotune.load_table(str(p)) == 3
    assert _lib.lib.vkc_gemm_tune_clear() == _lib.OK
    autotune.load_table()   # restore the shipped table
    assert autotune.bucket(1) == 0 and autotune.bucket(784) == 10 and autotune.bucket(1024) == 10


def test_grouped_entry_points_validate_without_gpu():
    """The one-launch-per-step entry points reject a missing device and bad
    arguments before touching the GPU."""
    import ctypes as C
    from vulkpy_gb300 import _lib
    L = _lib.lib
    ptrs = (C.c_void_p * 1)(None)
    n = (C.c_int64 * 1)(4)
    assert L.vkc_fill_f32_grouped(None, ptrs, n, 0.0, 1) == _lib.ERR_INVALID
    assert L.vkc_adam_update_grouped(None, ptrs, ptrs, ptrs, ptrs, ptrs, n, 1, 1e-3, 0.9, 0.999, 1e-8) \
        == _lib.ERR_INVALID
    assert L.vkc_sgd_update_grouped(None, ptrs, ptrs, n, 1e-2, 1) == _lib.ERR_INVALID
    s, t = C.c_int(), C.c_int()
    assert L.vkc_gemm_plan_get(None, _lib.MM_BF16X3, 256, 1024, 784, C.byref(s), C.byref(t)) == _lib.ERR_INVALID


def test_injected_host_allocation_failure_without_gpu():
    """The allocation error path is testable on the host: an injected failure
    returns VKC_ERR_OOM before any CUDA call, counts as an allocation
    request, and switches itself off after firing."""
    import ctypes as C
    from vulkpy_gb300 import _lib
    L = _lib.lib
    c0, c1 = C.c_uint64(), C.c_uint64()
    assert L.vkc_alloc_count(C.byref(c0)) == _lib.OK
    p = C.c_void_p()
    try:
        assert L.vkc_inject_alloc_failure(0) == _lib.OK
        assert L.vkc_host_alloc(4096, C.byref(p)) == _lib.ERR_OOM and not p.value
        assert "injected allocation failure" in _lib.last_error()
    finally:
        L.vkc_inject_alloc_failure(-1)
    assert L.vkc_alloc_count(C.byref(c1)) == _lib.OK and c1.value == c0.value + 1
    assert L.vkc_alloc_count(None) == _lib.ERR_INVALID
