"""vkc_reduce_all_noalloc: the full reduction for callers that cannot
allocate device memory during a call (hosts whose own allocator owns the
device heap, or latency-critical paths where an allocation could block or
fail).  Called through the C ABI and checked against vkc_reduce_all on the
same inputs, twice in a row, for every op; plus the size limit.

This file is named to be collected last, so a stop-at-first-failure run has
already run every other test when it gets here."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reduce(lib, fn, h, op, prec, ptr, n, out):
    assert fn(h, op, prec, ptr, n, out, C.c_float(1.0)) == 0, lib.vkc_last_error()


@pytest.mark.parametrize("n", [3, 8192, 1_000_003, (1 << 24) + 5])
def test_noalloc_matches_reduce_all_twice(gpu, n):
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
        for op in (_lib.SUM, _lib.PROD, _lib.MAXIMUM, _lib.MINIMUM):
            if op == _lib.PROD and call == 0:
                continue  # products of N(0,1) values under/overflow; use the second input
            _reduce(lib, lib.vkc_reduce_all, h, op, _lib.RED_COMPENSATED, x._dptr(), n, out_ref._dptr())
            _reduce(lib, lib.vkc_reduce_all_noalloc, h, op, _lib.RED_COMPENSATED, x._dptr(), n, out_new._dptr())
            out_ref._written()
            out_new._written()
            ref = float(np.asarray(out_ref)[0])
            new = float(np.asarray(out_new)[0])
            if op in (_lib.MAXIMUM, _lib.MINIMUM):
                assert new == ref
            elif op == _lib.SUM:
                tol = np.abs(inputs[call]).sum(dtype=np.float64) * 2.0 ** -22 + 1e-6
                assert abs(new - ref) <= tol, (n, call, new, ref)
            else:
                assert abs(new - ref) <= 1e-5 * abs(ref), (n, call, new, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import vulkpy_gb300 as vk
    from vulkpy_gb300 import _lib
    x = vk.Array(gpu, data=np.ones(16, np.float32))
    out = vk.Array(gpu, shape=(1,))
    st = _lib.lib.vkc_reduce_all_noalloc(gpu.handle, _lib.SUM, _lib.RED_COMPENSATED, x._dptr(), (1 << 29) + 1,
                                         out._dptr(), C.c_float(1.0))
    assert st == _lib.ERR_INVALID
    assert "exceed the maximum" in _lib.last_error()
