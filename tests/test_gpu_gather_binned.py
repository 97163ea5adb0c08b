"""The binned form of the flat gather (indices partitioned by table window,
each window read while it is in L2, values put back in order) against numpy
and against the direct kernel: bit-exact (a gather copies values).  Cases:
partial last chunks, one-element chunks, every index in one window, indices
out of range (NaN and bit0 of the error word, as the direct kernel), an empty
table, and tables just past the size at which the form is chosen by itself.
"""
import numpy as np
import pytest

from oracle import ops as O
from vulkpy_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


def _gather(vk, gpu, table, idx, mode):
    _lib.lib.vkc_set_gather_bins(mode)
    try:
        return np.asarray(table.gather(vk.U32Array(gpu, data=idx)))
    finally:
        _lib.lib.vkc_set_gather_bins(0)   # the default


@pytest.mark.parametrize("n_a,n_idx", [(1000, 1), (1000, 4096), (1000, 4097), (70000, 3 * 4096 + 123),
                                        ((1 << 21) + 3, 20000), ((1 << 22) + 5, 9 * 4096)])
def test_binned_matches_direct_and_numpy(gpu, vk, n_a, n_idx):
    rng = np.random.default_rng(n_a + n_idx)
    a = rng.standard_normal(n_a).astype(np.float32)
    idx = rng.integers(0, n_a, size=n_idx, dtype=np.uint32)
    table = vk.Array(gpu, data=a)
    got = _gather(vk, gpu, table, idx, 2)
    np.testing.assert_array_equal(got, O.gather(a, idx))
    np.testing.assert_array_equal(got, _gather(vk, gpu, table, idx, 1))
    assert gpu.check_errors() == 0


def test_binned_one_window_and_repeats(gpu, vk):
    """All indices in one window (one non-empty run per chunk) and every
    index repeated many times."""
    a = np.arange(1 << 22, dtype=np.float32)
    table = vk.Array(gpu, data=a)
    idx = np.repeat(np.arange(7, dtype=np.uint32) * 1000 + 5, 4096 * 3 // 7 + 1)[: 4096 * 3 + 17]
    np.testing.assert_array_equal(_gather(vk, gpu, table, idx, 2), a[idx])
    idx = (np.arange(5 * 4096, dtype=np.uint32) % 64) + (1 << 21)
    np.testing.assert_array_equal(_gather(vk, gpu, table, idx, 2), a[idx])
    assert gpu.check_errors() == 0


def test_binned_out_of_range_sets_flag(gpu, vk):
    gpu.check_errors()  # clear
    rng = np.random.default_rng(3)
    n_a = 50000
    a = rng.standard_normal(n_a).astype(np.float32)
    idx = rng.integers(0, n_a, size=2 * 4096 + 9, dtype=np.uint32)
    bad = rng.choice(idx.size, size=300, replace=False)
    idx[bad] = rng.integers(n_a, 1 << 32, size=bad.size, dtype=np.uint64).astype(np.uint32)
    idx[-1] = 0xFFFFFFFF
    got = _gather(vk, gpu, vk.Array(gpu, data=a), idx, 2)
    ok = idx < n_a
    np.testing.assert_array_equal(got[ok], a[idx[ok]])
    assert np.isnan(got[~ok]).all()
    assert gpu.check_errors() & 1
    assert gpu.check_errors() == 0
    # every index out of range, and a table of one element
    got = _gather(vk, gpu, vk.Array(gpu, data=np.ones(1, np.float32)), np.full(5000, 7, np.uint32), 2)
    assert np.isnan(got).all() and gpu.check_errors() & 1


def test_binned_chosen_by_size(gpu, vk):
    """A 2^25-float table and 2^21 + 3 indices take the binned form by
    default; the values equal the direct kernel's."""
    rng = np.random.default_rng(11)
    n_a = 1 << 25
    a = rng.standard_normal(n_a).astype(np.float32)
    idx = rng.integers(0, n_a, size=(1 << 21) + 3, dtype=np.uint32)
    table = vk.Array(gpu, data=a)
    got = _gather(vk, gpu, table, idx, 0)
    np.testing.assert_array_equal(got, a[idx])
    np.testing.assert_array_equal(got, _gather(vk, gpu, table, idx, 1))
    assert gpu.check_errors() == 0


def test_gather_bins_mode_is_checked():
    assert _lib.lib.vkc_set_gather_bins(3) != 0
    assert _lib.lib.vkc_set_gather_bins(0) == 0
