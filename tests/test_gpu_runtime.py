"""Runtime behaviour on the GPU: host mirror semantics, job waits and
timeouts, error reporting, and calls made directly through the C ABI."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


def test_host_writes_and_reads_follow_program_order(gpu, vk):
    a = vk.Array(gpu, data=np.arange(6, dtype=np.float32))
    b = a * 2.0
    a[1] = 100.0                 # host write after a device read of a
    c = a + 1.0                  # must see the write
    np.testing.assert_array_equal(np.asarray(b), np.arange(6) * 2.0)
    np.testing.assert_array_equal(np.asarray(c), [1, 101, 3, 4, 5, 6])
    a += 1.0                     # device write invalidates the host copy
    assert np.asarray(a)[1] == 101.0
    a.array[0] = -5.0            # writes through .array reach the device
    np.testing.assert_array_equal(np.asarray(a * 1.0)[:2], [-5.0, 101.0])
    view = np.asarray(a)
    assert not view.flags.writeable


def test_large_pinned_mirror_roundtrip(gpu, vk):
    x = np.random.default_rng(0).standard_normal((1024, 1024)).astype(np.float32)
    a = vk.Array(gpu, data=x)
    a[:, 3] = 7.0
    b = a + 0.0
    x[:, 3] = 7.0
    np.testing.assert_array_equal(np.asarray(b), x)


def test_reshape_and_errors(gpu, vk):
    a = vk.Array(gpu, data=[1, 2, 3, 4])
    a.reshape((2, 2))
    np.testing.assert_array_equal(np.asarray(a), [[1, 2], [3, 4]])
    with pytest.raises(ValueError):
        a.reshape((3, 2))
    with pytest.raises(ValueError):
        vk.Array(gpu, data=[1, 1]) + vk.Array(gpu, data=[1, 1, 1])
    with pytest.raises(ValueError):
        vk.Array(gpu, data=[1.0, 2.0, 3.0]).broadcast_to((4,))
    with pytest.raises(ValueError):
        vk.Array(gpu)
    with pytest.raises(ValueError):
        vk.random.Xoshiro128pp(gpu).randrange(shape=(3,), low=5, high=5)


def test_zero_fill_and_empty(gpu, vk):
    z = vk.zeros(gpu, shape=(3, 5))
    np.testing.assert_array_equal(np.asarray(z), np.zeros((3, 5)))
    e = vk.Array(gpu, shape=(0, 4))
    f = e + 1.0
    assert np.asarray(f).shape == (0, 4)


def test_job_wait_timeout_then_complete(gpu, vk):
    n = 4096
    a = vk.Array(gpu, data=np.ones((n, n), dtype=np.float32))
    gpu.wait()
    c = a @ a                     # ~0.1 s of fp32 work queued
    with pytest.raises(RuntimeError, match="Timeout at Command Wait"):
        c.job.wait(timeout_ns=1000)
    c.wait()
    assert np.asarray(c)[0, 0] == n


def test_gpu_equality_and_shared_device(gpu, vk):
    assert vk.GPU() == gpu
    assert (gpu == 1) is False


def test_c_abi_direct_calls(gpu):
    """Allocate, upload, compute and read back through the C ABI only,
    including a 4-byte-offset (unaligned) pointer path."""
    from vulkpy_gb300 import _lib
    lib, h = _lib.lib, gpu.handle
    n = 1001
    x = np.arange(n, dtype=np.float32)
    d_x, d_y = C.c_void_p(), C.c_void_p()
    assert lib.vkc_upload(h, x.ctypes.data, x.nbytes, C.byref(d_x)) == 0
    assert lib.vkc_alloc(h, (n + 4) * 4, C.byref(d_y)) == 0
    assert lib.vkc_binary_scalar(h, _lib.MUL, d_x.value + 4, 3.0, d_y.value + 4, n - 1) == 0
    y = np.empty(n - 1, np.float32)
    assert lib.vkc_d2h(h, y.ctypes.data, d_y.value + 4, y.nbytes) == 0
    np.testing.assert_array_equal(y, x[1:] * 3)
    st = lib.vkc_reduce_axis(h, 99, d_x, 1, n, 1, d_y, 0, C.c_float(1.0))
    assert st == _lib.ERR_INVALID and "unknown reduce op" in _lib.last_error()
    assert lib.vkc_free(h, d_x) == 0 and lib.vkc_free(h, d_y) == 0
    j = C.c_void_p()
    assert lib.vkc_job_record(h, C.byref(j)) == 0
    assert lib.vkc_job_wait(j, -1) == 0
    done = C.c_int()
    assert lib.vkc_job_query(j, C.byref(done)) == 0 and done.value == 1
    assert lib.vkc_job_destroy(j) == 0


def test_graph_collected_during_another_capture(gpu, vk):
    """A launched graph that the garbage collector destroys while another
    graph is being captured must not invalidate that capture; it is
    destroyed (and its memory freed) once the capture ends."""
    import gc
    x = vk.Array(gpu, data=np.arange(4096, dtype=np.float32))
    gc.collect()
    gc.disable()
    try:
        old = vk.graph.Graph(gpu)
        with old:
            y = (x + 1.0) * 2.0
        old.launch()
        np.testing.assert_array_equal(np.asarray(y), (np.arange(4096, dtype=np.float32) + 1.0) * 2.0)
        cycle = {"g": old, "y": y}
        cycle["self"] = cycle
        del old, y, cycle
        g = vk.graph.Graph(gpu)
        with g:
            z = x * 3.0
            gc.collect()                      # destroys `old` mid-capture
            assert len(gpu._dev.zombies) == 1
            with gpu.branch():
                w = x - 1.0
            z = z + w
        assert gpu._dev.zombies == []
    finally:
        gc.enable()
    g.launch()
    np.testing.assert_array_equal(np.asarray(z), np.arange(4096, dtype=np.float32) * 4.0 - 1.0)
    g.launch()
    np.testing.assert_array_equal(np.asarray(z), np.arange(4096, dtype=np.float32) * 4.0 - 1.0)


def test_graph_output_tracked_when_python_reuses_ids(gpu, vk):
    """An array written by the captured ops may get the id() of a temporary
    freed earlier in the capture; every launch must still invalidate its
    host copy (otherwise reads after the second launch are stale)."""
    base = np.arange(1024, dtype=np.float32)
    x = vk.Array(gpu, data=base)
    g = vk.graph.Graph(gpu)
    ids = set()
    with g:
        for _ in range(20):
            t = x * 2.0
            ids.add(id(t))
            del t
        out = x + 1.0
    reused = id(out) in ids
    for k in range(4):
        x[:] = base * (k + 1)
        g.launch(flush=[x])
        np.testing.assert_array_equal(np.asarray(out), base * (k + 1) + 1.0, err_msg=f"launch {k}, reused={reused}")
