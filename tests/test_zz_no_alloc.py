"""vkc_reduce_all_noalloc: the full reduction for callers that cannot
allocate device memory during a call (hosts whose own allocator owns the
device heap, or latency-critical paths where an allocation could block or
fail).  Called through the C ABI and checked, twice in a row for every op:
  * against vkc_reduce_all on the same inputs: the same bits (both entry
    points launch the same grid);
  * against float64 truth: |err| <= 2^-22 sum|x| for sums, rel 1e-5 for
    products, exact for maximum / minimum;
  * for allocating nothing: the library's allocation counter and the
    device's free memory are unchanged across the call.
Plus the size limit.

This file is named to be collected last, so a stop-at-first-failure run has
already run every other test when it gets here."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reduce(lib, fn, h, op, prec, ptr, n, out):
    assert fn(h, op, prec, ptr, n, out, C.c_float(1.0)) == 0, lib.vkc_last_error()


def _alloc_count(lib):
    c = C.c_uint64()
    assert lib.vkc_alloc_count(C.byref(c)) == 0
    return c.value


@pytest.mark.parametrize("n", [3, 8192, 1_000_003, (1 << 24) + 5])
def test_noalloc_matches_reduce_all_twice(gpu, n):
    import torch
    import vulkpy_gb300 as vk
    from vulkpy_gb300 import _lib
    lib, h = _lib.lib, gpu.handle
    rng = np.random.default_rng(n)
    inputs = [rng.standard_normal(n).astype(np.float32),
              rng.uniform(0.9999, 1.0001, n).astype(np.float32)]
    out_ref = vk.Array(gpu, shape=(1,))
    out_new = vk.Array(gpu, shape=(1,))
    for call in range(2):  # two calls in a row share the static scratch
        x = vk.Array(gpu, data=inputs[call])
        x64 = inputs[call].astype(np.float64)
        for op in (_lib.SUM, _lib.PROD, _lib.MAXIMUM, _lib.MINIMUM):
            if op == _lib.PROD and call == 0:
                continue  # products of N(0,1) values under/overflow; use the second input
            _reduce(lib, lib.vkc_reduce_all, h, op, _lib.RED_COMPENSATED, x._dptr(), n, out_ref._dptr())
            gpu.wait()
            before = _alloc_count(lib)
            free_before = torch.cuda.mem_get_info(0)[0]
            _reduce(lib, lib.vkc_reduce_all_noalloc, h, op, _lib.RED_COMPENSATED, x._dptr(), n, out_new._dptr())
            gpu.wait()
            assert _alloc_count(lib) == before
            assert torch.cuda.mem_get_info(0)[0] == free_before
            out_ref._written()
            out_new._written()
            ref = float(np.asarray(out_ref)[0])
            new = float(np.asarray(out_new)[0])
            assert np.float32(new).tobytes() == np.float32(ref).tobytes(), (n, call, op, new, ref)
            if op == _lib.MAXIMUM:
                assert new == x64.max()
            elif op == _lib.MINIMUM:
                assert new == x64.min()
            elif op == _lib.SUM:
                tol = np.abs(x64).sum() * 2.0 ** -22 + 1e-6
                assert abs(new - x64.sum()) <= tol, (n, call, new)
            else:
                assert abs(new - np.prod(x64)) <= 1e-5 * abs(np.prod(x64)), (n, call, new)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import vulkpy_gb300 as vk
    from vulkpy_gb300 import _lib
    x = vk.Array(gpu, data=np.ones(16, np.float32))
    out = vk.Array(gpu, shape=(1,))
    st = _lib.lib.vkc_reduce_all_noalloc(gpu.handle, _lib.SUM, _lib.RED_COMPENSATED, x._dptr(), (1 << 29) + 1,
                                         out._dptr(), C.c_float(1.0))
    assert st == _lib.ERR_INVALID
    assert "exceed the maximum" in _lib.last_error()
