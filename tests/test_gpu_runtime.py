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


def test_enable_debug_raises_at_the_failing_op(gpu, vk):
    """util.enable_debug (vulkpy/util.py:19-54 turns on Vulkan validation
    layers): here every op synchronises and reads the device error word, so
    an out-of-range gather raises at that op rather than silently writing
    NaN; the ops before and after it run normally."""
    a = vk.Array(gpu, data=np.arange(10, dtype=np.float32))
    good = vk.U32Array(gpu, data=[1, 2, 3])
    bad = vk.U32Array(gpu, data=[1, 10, 3])
    gpu.check_errors()
    vk.util.enable_debug(api_dump=False)
    try:
        assert vk.util.debug_enabled()
        np.testing.assert_array_equal(np.asarray(a.gather(good)), [1, 2, 3])
        with pytest.raises(IndexError, match="gather index out of range"):
            a.gather(bad)
        np.testing.assert_array_equal(np.asarray(a + 1.0)[:2], [1, 2])
    finally:
        vk.util.disable_debug()
    assert not vk.util.debug_enabled()
    out = a.gather(bad)              # without debug: NaN and the flag, no exception
    assert np.isnan(np.asarray(out)[1])
    assert gpu.check_errors() & 1


def test_injected_allocation_failures_raise_and_recover(gpu, vk):
    """Allocation failures injected on the host (vkc_inject_alloc_failure,
    no GPU fault): an array allocation, an upload, a pinned host buffer and
    an op's internal scratch each fail with MemoryError at the call that
    allocates, and the device keeps working afterwards."""
    from vulkpy_gb300 import _lib
    lib = _lib.lib
    x = vk.Array(gpu, data=np.ones((256, 256), dtype=np.float32))
    try:
        assert lib.vkc_inject_alloc_failure(0) == 0
        with pytest.raises(MemoryError, match="injected allocation failure"):
            vk.Array(gpu, shape=(1000,))
        assert lib.vkc_inject_alloc_failure(0) == 0
        with pytest.raises(MemoryError, match="injected allocation failure"):
            vk.Array(gpu, data=np.ones(1000, dtype=np.float32))
        p = C.c_void_p()
        assert lib.vkc_inject_alloc_failure(0) == 0
        assert lib.vkc_host_alloc(1 << 20, C.byref(p)) == _lib.ERR_OOM and not p.value
        assert "injected" in _lib.last_error()
        # the second allocation of a bf16 matmul is its operand scratch (the
        # first is the result array)
        assert lib.vkc_inject_alloc_failure(1) == 0
        with pytest.raises(MemoryError, match="injected allocation failure"):
            vk.vkarray.matmul(x, x, precision="bf16")
    finally:
        lib.vkc_inject_alloc_failure(-1)
    c = vk.vkarray.matmul(x, x, precision="bf16")
    np.testing.assert_allclose(np.asarray(c), np.full((256, 256), 256.0), rtol=1e-6)
    assert gpu.check_errors() == 0


def test_async_pinned_upload_and_prefetch(gpu, vk):
    """Array(data=pinned) returns once the copy is queued; ops on the array
    wait for it on the device.  prefetch() starts the read-back without
    waiting; a read after it returns the values of the ops issued before it,
    and a write after it makes the prefetched copy stale (not used)."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal((1024, 1024)).astype(np.float32)
    xp = vk.vkarray.empty_pinned(x.shape)
    xp[...] = x
    a = vk.Array(gpu, data=xp)
    b = a * 2.0
    a.wait()                       # the upload is done: the source may change
    xp[...] = 0.0
    np.testing.assert_array_equal(np.asarray(b), x * 2.0)
    np.testing.assert_array_equal(np.asarray(a), x)
    c = a + 1.0
    c.prefetch()
    d = c * 3.0                    # issued after the prefetch, reads c
    np.testing.assert_array_equal(np.asarray(c), x + 1.0)
    np.testing.assert_array_equal(np.asarray(d), (x + 1.0) * 3.0)
    c.prefetch()                   # already on the host: nothing to do
    e = a - 1.0
    e.prefetch()
    e += 10.0                      # written after the prefetch
    np.testing.assert_array_equal(np.asarray(e), (x - 1.0) + 10.0)
    f = a * 0.5
    f.prefetch()
    del f                          # dropped with its read-back in flight
    gpu.wait()


def test_pipelined_steps_match_serial(gpu, vk):
    """The pipelined loop of the end-to-end benchmark (issue step i+1 before
    reading step i's prefetched results) gives the serial loop's values."""
    rng = np.random.default_rng(6)
    hs = [rng.standard_normal((512, 2048)).astype(np.float32) for _ in range(4)]
    row = rng.uniform(0.5, 2, (1, 2048)).astype(np.float32)
    r = vk.Array(gpu, data=row)

    def step(h):
        X = vk.Array(gpu, data=h)
        X *= r
        s = X.sum(axis=1)
        m = X.maximum(axis=0)
        return [s, m, X]

    serial = [[np.asarray(o).copy() for o in step(h)] for h in hs]
    pins = []
    for h in hs:
        p = vk.vkarray.empty_pinned(h.shape)
        p[...] = h
        pins.append(p)
    got, pending = [], None
    for p in pins + [None]:
        cur = None
        if p is not None:
            cur = step(p)
            for o in cur:
                o.prefetch()
        if pending is not None:
            got.append([np.asarray(o).copy() for o in pending])
        pending = cur
    for a, b in zip(serial, got):
        for u, v in zip(a, b):
            np.testing.assert_array_equal(u, v)


def test_upload_buffers_are_reused_after_their_last_use(gpu, vk):
    """A freed upload buffer (>= 1 MiB) is cached with an event after its
    last use on the compute stream; an upload of the same size takes it
    without allocating once that use has finished, and allocates instead
    while it is still queued.  Results of ops queued on old contents stay
    correct either way."""
    from vulkpy_gb300 import _lib
    rng = np.random.default_rng(11)
    n = 1 << 22                                   # 16 MiB of float32
    hosts = [rng.standard_normal(n).astype(np.float32) for _ in range(6)]
    pins = []
    for h in hosts:
        p_ = vk.vkarray.empty_pinned(h.shape)
        p_[...] = h
        pins.append(p_)

    def allocs():
        c = C.c_uint64()
        assert _lib.lib.vkc_alloc_count(C.byref(c)) == 0
        return c.value

    outs = []
    a = vk.Array(gpu, data=pins[0])
    for i in range(1, 6):
        y = a
        for _ in range(8):                        # queue work that reads the buffer
            y = y * 1.5 + 1.0
        outs.append(y)
        del a, y
        if i % 2:
            gpu.wait()                            # the last use has finished: reused
            before = allocs()
            a = vk.Array(gpu, data=pins[i])
            assert allocs() == before, "a finished cached upload buffer should have been reused"
        else:
            a = vk.Array(gpu, data=pins[i])       # maybe still queued: either way correct
    outs.append(a * 1.0)
    for i, o in enumerate(outs[:5]):
        exp = hosts[i].astype(np.float32)
        for _ in range(8):
            exp = exp * np.float32(1.5) + np.float32(1.0)
        np.testing.assert_array_equal(np.asarray(o), exp)
    np.testing.assert_array_equal(np.asarray(outs[5]), hosts[5])


def test_whole_array_assignment_uploads_in_place(gpu, vk):
    """a[:] = host array (pageable or pinned, same shape) overwrites the
    device buffer with one copy ordered after the ops already queued on it:
    those see the old contents, later ops the new; no read-back happens."""
    rng = np.random.default_rng(3)
    x, y, z = (rng.standard_normal((512, 300)).astype(np.float32) for _ in range(3))
    a = vk.Array(gpu, data=x)
    b = a * 2.0                         # queued on the old contents
    a[:] = y                            # pageable
    c = a + 1.0
    zp = vk.vkarray.empty_pinned(z.shape)
    zp[...] = z
    a.prefetch()                        # a read-back in flight before the next overwrite
    a[...] = zp                         # pinned
    d = a * 3.0
    np.testing.assert_array_equal(np.asarray(b), x * np.float32(2.0))
    np.testing.assert_array_equal(np.asarray(c), y + np.float32(1.0))
    np.testing.assert_array_equal(np.asarray(d), z * np.float32(3.0))
    np.testing.assert_array_equal(np.asarray(a), z)
    a[:] = x.astype(np.float64)         # converted to float32 first
    np.testing.assert_array_equal(np.asarray(a), x)
    a[:, 0] = 5.0                       # partial writes still go through the host mirror
    exp = x.copy()
    exp[:, 0] = 5.0
    np.testing.assert_array_equal(np.asarray(a * 1.0), exp)
