"""
Array engine (drop-in for vulkpy.vkarray, vulkpy/vkarray.py:1-1542).

* :class:`GPU` -- one CUDA device, shared by every ``GPU(idx)`` object with
  the same index; all ops run in order on its compute stream.
* :class:`Array` (float32) / :class:`U32Array` (uint32) -- device buffers.

Differences in mechanism (the API and results follow the reference):

* The reference keeps every buffer in host-visible mapped memory and lets
  Python read it through a live numpy view (vkarray.py:236-237, 430-431).
  Here data lives in HBM.  Each array has a host *mirror* that is filled
  lazily: a host read waits for the array's last op and copies it back
  once; a host write marks the mirror as the newest copy and it is uploaded
  before the next op that uses the array.  Reads never race with pending
  GPU work (the reference's ``__setitem__`` does, vkarray.py:176-177).
* ``job`` is a marker of the op that produced the array; ``wait()`` blocks
  only the host.  Dependent ops need no waits: they are ordered on the
  stream (the reference host-waits per dependency, _vkarray.cc:430-432).
  Memory is freed stream-ordered, so ``_keep`` is not needed to keep inputs
  alive; the attribute exists for compatibility.
"""
from __future__ import annotations

import ctypes as C
import functools
import logging
import os
import threading
from typing import Iterable, List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _lib
from ._lib import lib, check, shape_arg
from .util import debug_enabled
from .vktyping import KeyType, ValueType, Resource, ArrayProtocol

__all__ = ["GPU", "U32Array", "Shape", "Array", "zeros", "Job"]

logger = logging.getLogger("vulkpy_gb300")

_PINNED_MIN_BYTES = 1 << 20  # host mirrors from 1 MiB up use pinned memory

_MATMUL_PRECISION = {"fp32": _lib.MM_FP32, "bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}


# ---------------------------------------------------------------- devices


class _Device:
    """An opened CUDA device: handle, op sequence numbers, error checks."""

    _cache: dict = {}
    _lock = threading.Lock()

    def __init__(self, idx: int, priority: float):
        h = C.c_void_p()
        check(lib.vkc_device_open(int(idx), float(priority), C.byref(h)))
        self.h = h
        self.idx = idx
        self.seq = 0        # ops issued
        self.done = 0       # ops known to be complete
        self.capture = None  # the Graph being captured on this device, if any
        self.streams = [None]  # stack of current streams (None: the device's own)
        self.spare = []        # side streams for branches
        self.deferred = []     # (ptr, graph) frees held back while branches are open
        self.zombies = []      # (graph handle, its allocations) dropped during a capture
        sm = C.c_int()
        name = C.create_string_buffer(256)
        check(lib.vkc_device_info(h, C.byref(sm), name, 256))
        self.sm_count = sm.value
        self.name = name.value.decode()

    @classmethod
    def get(cls, idx: int, priority: float) -> "_Device":
        with cls._lock:
            d = cls._cache.get(idx)
            if d is None:
                d = cls._cache[idx] = _Device(idx, priority)
            return d

    def issued(self) -> "Job":
        self.seq += 1
        if debug_enabled():
            self.synchronize()
            flags = C.c_uint32()
            check(lib.vkc_device_check_errors(self.h, C.byref(flags)))
            if flags.value & 1:
                raise IndexError("gather index out of range")
            if flags.value & 2:
                raise RuntimeError("tensor-core GEMM pipeline wait timed out")
        return Job(self, self.seq)

    def wait_seq(self, seq: int, timeout_ns: Optional[int] = None):
        if seq <= self.done:
            return
        target = self.seq
        j = C.c_void_p()
        check(lib.vkc_job_record(self.h, C.byref(j)))
        try:
            check(lib.vkc_job_wait(j, -1 if timeout_ns is None else int(timeout_ns)))
        finally:
            lib.vkc_job_destroy(j)
        self.done = max(self.done, target)

    def synchronize(self):
        target = self.seq
        check(lib.vkc_device_synchronize(self.h))
        self.done = max(self.done, target)

    # -- freeing ------------------------------------------------------------
    def release(self, ptr: int, graph) -> None:
        """Free a device buffer, stream-ordered, respecting open branches and
        graph captures (see _DevBuf)."""
        if graph is not None and self.capture is not graph:
            return                                  # owned by its graph
        if len(self.streams) > 1:                   # a branch is open
            self.deferred.append((ptr, graph))
            return
        cap = self.capture
        if cap is not None and graph is not cap:    # older buffer: after the capture
            cap._deferred.append(ptr)
            return
        if graph is not None:
            graph._allocated.discard(ptr)
        lib.vkc_free(self.h, ptr)

    def reap(self) -> None:
        """Destroy graphs (and free their memory) that were dropped while a
        capture or a branch was open; a no-op until neither is."""
        if self.capture is not None or len(self.streams) > 1:
            return
        while self.zombies:
            h, ptrs = self.zombies.pop()
            if h is not None:
                lib.vkc_graph_destroy(h)
            for p in ptrs:
                lib.vkc_free(self.h, p)

    # -- branches -----------------------------------------------------------
    def own_stream(self) -> bool:
        """True when work goes to the device's own stream (no branch open)."""
        return len(self.streams) == 1

    def branch_enter(self):
        parent = self.streams[-1]
        if self.spare:
            s = self.spare.pop()
        else:
            p = C.c_void_p()
            check(lib.vkc_stream_create(self.h, C.byref(p)))
            s = p.value
        check(lib.vkc_stream_wait(self.h, s, parent))      # fork
        check(lib.vkc_device_set_stream(self.h, s))
        self.streams.append(s)

    def branch_exit(self):
        s = self.streams.pop()
        parent = self.streams[-1]
        check(lib.vkc_device_set_stream(self.h, parent))
        check(lib.vkc_stream_wait(self.h, parent, s))      # join
        self.spare.append(s)
        if len(self.streams) == 1:
            pending, self.deferred = self.deferred, []
            for ptr, graph in pending:
                self.release(ptr, graph)
            self.reap()


class Job:
    """Completion marker of one op (replaces vulkpy's Job, _vkarray.cc:392-457)."""

    __slots__ = ("_dev", "seq")

    def __init__(self, dev: _Device, seq: int):
        self._dev = dev
        self.seq = seq

    def wait(self, timeout_ns: Optional[int] = None):
        """Block until the op is done; raises RuntimeError
        ("Timeout at Command Wait") when ``timeout_ns`` passes first."""
        self._dev.wait_seq(self.seq, timeout_ns)

    def done(self) -> bool:
        return self.seq <= self._dev.done


class GPU:
    """
    GPU instance (vulkpy/vkarray.py:68-137).

    Examples
    --------
    >>> import vulkpy_gb300 as vk
    >>> gpu = vk.GPU()
    >>> gpu == vk.GPU()
    True
    """

    def __init__(self, idx: int = 0, priority: float = 0.0):
        self._idx = idx
        self._dev = _Device.get(idx, priority)
        # Warp-level reductions are always available on CUDA devices.
        self.canSubgroupArithmetic = True
        self.matmul_precision = os.environ.get("VULKPY_GB300_MATMUL", "fp32")
        self.reduce_precision = _lib.RED_COMPENSATED
        logger.info(f"GPU {idx}: {self._dev.name}, {self._dev.sm_count} SMs")

    def __eq__(self, other: object):
        if not isinstance(other, GPU):
            return NotImplemented
        return self._idx == other._idx

    __hash__ = None  # like the reference (defines __eq__ only)

    @property
    def handle(self):
        return self._dev.h

    def flush(self, arrays: Iterable["_GPUArray"]):
        """Upload host-side writes of ``arrays`` now (normally done lazily)."""
        for a in arrays:
            a._ensure_device()

    def wait(self):
        """Wait for all GPU operations (GPU.wait, _vkarray.cc:560-562)."""
        self._dev.synchronize()

    def branch(self):
        """Context manager: ops inside run on a side stream that forks from the
        current stream at entry and joins it at exit, so independent branches
        (e.g. one per model) run concurrently; inside a graph capture they
        become parallel branches of the graph.  Buffers released while a
        branch is open are freed after the join."""
        gpu = self

        class _Branch:
            def __enter__(self):
                gpu._dev.branch_enter()
                return self

            def __exit__(self, *exc):
                gpu._dev.branch_exit()
                return False

        return _Branch()

    def check_errors(self) -> int:
        """Read and clear the device error word (bit0: gather index out of range)."""
        flags = C.c_uint32()
        check(lib.vkc_device_check_errors(self._dev.h, C.byref(flags)))
        return flags.value


# ---------------------------------------------------------------- memory


class _PinnedPool:
    """Free lists of pinned host blocks by power-of-two capacity."""

    def __init__(self, limit_bytes: int = 8 << 30):
        self.free: dict = {}
        self.cached = 0
        self.limit = limit_bytes
        self.lock = threading.Lock()
        self.allocs = 0  # blocks allocated from the driver (misses)

    def get(self, nbytes: int) -> Tuple[int, int]:
        cap = 1 << max(20, (nbytes - 1).bit_length())
        with self.lock:
            lst = self.free.get(cap)
            if lst:
                self.cached -= cap
                return lst.pop(), cap
        p = C.c_void_p()
        check(lib.vkc_host_alloc(cap, C.byref(p)))
        self.allocs += 1
        return p.value, cap

    def put(self, ptr: int, cap: int):
        with self.lock:
            if self.cached + cap <= self.limit:
                self.free.setdefault(cap, []).append(ptr)
                self.cached += cap
                return
        lib.vkc_host_free(ptr)


_pinned_pool = _PinnedPool()


class _PinnedBlock:
    """Owner of one pinned block; numpy views keep it alive via ``base``."""

    def __init__(self, nbytes: int, shape, dtype):
        self.ptr, self.cap = _pinned_pool.get(nbytes)
        self.__array_interface__ = {
            "shape": tuple(shape), "typestr": np.dtype(dtype).str,
            "data": (self.ptr, False), "version": 3,
        }

    def __del__(self):
        try:
            _pinned_pool.put(self.ptr, self.cap)
        except Exception:  # interpreter shutdown
            pass


def empty_pinned(shape, dtype=np.float32) -> np.ndarray:
    """Uninitialised numpy array in pinned (page-locked) host memory.

    ``Array(gpu, data=a)`` from such an array uploads by DMA at full link
    speed and returns as soon as the copy is queued (the GPU's later ops on
    the new array wait for it on the device): leave ``a`` unchanged until the
    upload is done -- ``wait()`` on the new array, or any host access to
    it, waits for that.  The block returns to a pool when the array is
    garbage collected."""
    nbytes = max(1, int(np.prod(shape, dtype=np.int64))) * np.dtype(dtype).itemsize
    return np.asarray(_PinnedBlock(nbytes, tuple(shape), dtype))


def _is_pinned(a: np.ndarray) -> bool:
    """True when ``a``'s data lies in a block from ``empty_pinned``."""
    b = a
    while b is not None and not isinstance(b, _PinnedBlock):
        b = getattr(b, "base", None)
    if b is None:
        return False
    p = a.__array_interface__["data"][0]
    return b.ptr <= p and p + a.nbytes <= b.ptr + b.cap


def _host_buffer(shape, dtype) -> Tuple[np.ndarray, bool]:
    nbytes = int(np.prod(shape, dtype=np.int64)) * np.dtype(dtype).itemsize
    if nbytes >= _PINNED_MIN_BYTES:
        return np.asarray(_PinnedBlock(nbytes, shape, dtype)), True
    return np.empty(shape, dtype=dtype), False


class _DevBuf:
    """Device allocation, freed stream-ordered when garbage collected.

    While a graph is being captured on the device, new allocations become
    graph memory: freed inside the capture they are graph free nodes; still
    live at the end of the capture they belong to the graph (re-made at the
    same address on every launch, released when the graph is).  Frees of
    older buffers during a capture are deferred until it ends."""

    __slots__ = ("dev", "ptr", "nbytes", "graph", "h2d_job")

    def __init__(self, dev: _Device, nbytes: int, src: Optional[np.ndarray] = None, pinned: bool = False):
        self.dev = dev
        self.nbytes = nbytes
        self.graph = dev.capture
        self.h2d_job = None
        p = C.c_void_p()
        if src is not None and nbytes > 0 and pinned and self.graph is None:
            # pinned source: queued on the copy stream, no host wait
            j = C.c_void_p()
            check(lib.vkc_upload_async(dev.h, src.ctypes.data, nbytes, C.byref(p), C.byref(j)))
            self.h2d_job = j.value
        elif src is not None and nbytes > 0:
            check(lib.vkc_upload(dev.h, src.ctypes.data, nbytes, C.byref(p)))
        else:
            check(lib.vkc_alloc(dev.h, nbytes, C.byref(p)))
        self.ptr = p.value
        if self.graph is not None and self.ptr:
            self.graph._allocated.add(self.ptr)

    def __del__(self):
        try:
            if self.ptr:
                self.dev.release(self.ptr, self.graph)
        except Exception:  # interpreter shutdown
            pass


class _BufferInfo:
    """Stand-in for vulkpy's Buffer object: ``size()`` in elements."""

    __slots__ = ("_a",)

    def __init__(self, a):
        self._a = a

    def size(self) -> int:
        return self._a._size

    def info(self):
        return self._a

    def range(self):
        return self._a


# ---------------------------------------------------------------- arrays


def _prod(shape) -> int:
    n = 1
    for s in shape:
        n *= int(s)
    return n


class _GPUArray(Resource):
    _dtype = np.float32

    def __init__(self, gpu: GPU):
        self._gpu: GPU = gpu
        self.job: Optional[Job] = None
        self._keep: List[Resource] = []
        self._buf: Optional[_DevBuf] = None
        self._host: Optional[np.ndarray] = None
        self._host_pinned = False
        self._host_valid = False
        self._dev_valid = True
        self._h2d_job = None  # raw job handle of a pending pinned upload
        self._h2d_src = None  # the pinned source that upload reads
        self._d2h_job = None  # raw job handle of a pending read-back (prefetch)
        self._d2h_fresh = False  # no op has written the array since that read-back

    # -- construction helpers
    def _init_storage(self, shape, data: Optional[np.ndarray]):
        self.shape = tuple(int(s) for s in shape)
        self._size = _prod(self.shape)
        nbytes = self._size * 4  # float32 and uint32 elements
        pinned = data is not None and _is_pinned(data)
        self._buf = _DevBuf(self._gpu._dev, nbytes, data, pinned)
        if self._buf.h2d_job is not None:
            self._h2d_job, self._h2d_src = self._buf.h2d_job, data

    def __del__(self):
        try:
            if self._d2h_job is not None:
                # the copy still writes into the host mirror: let it finish
                # before the mirror can go back to the pinned pool
                j, self._d2h_job = self._d2h_job, None
                lib.vkc_job_wait(j, -1)
                lib.vkc_job_destroy(j)
            if self._h2d_job is not None:
                lib.vkc_job_destroy(self._h2d_job)
                self._h2d_job = None
        except Exception:  # interpreter shutdown
            pass

    # -- synchronisation
    def wait(self):
        """Wait for the last op that wrote this array (vkarray.py:153-161)."""
        if self.job is not None:
            self.job.wait()
            self.job = None
        self._wait_h2d()
        self._keep = []

    def prefetch(self):
        """Start copying this array to the host now, without waiting: the copy
        runs after every op issued so far, on a separate stream, so it
        overlaps the ops issued after it; a later host read (``np.asarray``,
        indexing) then only waits for the copy.  No counterpart in the
        reference, whose arrays live in host-visible memory."""
        if self._host_valid or self._size == 0 or self._d2h_job is not None:
            return
        dev = self._gpu._dev
        if dev.capture is not None:
            return
        self._ensure_device()
        if self._host is None or not self._host_pinned:
            self._host, self._host_pinned = np.asarray(_PinnedBlock(self._size * 4, self.shape, self._dtype)), True
        elif self._host.shape != self.shape:
            self._host = self._host.reshape(self.shape)
        j = C.c_void_p()
        check(lib.vkc_d2h_async(dev.h, self._host.ctypes.data, self._buf.ptr, self._buf.nbytes, C.byref(j)))
        self._d2h_job = j.value
        self._d2h_fresh = True

    def _wait_d2h(self):
        if self._d2h_job is not None:
            j, self._d2h_job = self._d2h_job, None
            try:
                check(lib.vkc_job_wait(j, -1))
            finally:
                lib.vkc_job_destroy(j)
            if self._d2h_fresh:
                self._host_valid = True
                self.job = None
                self._keep = []

    def flush(self):
        """Upload pending host-side writes now."""
        self._ensure_device()

    def _wait_h2d(self):
        if self._h2d_job is not None:
            j, self._h2d_job = self._h2d_job, None
            try:
                check(lib.vkc_job_wait(j, -1))
            finally:
                lib.vkc_job_destroy(j)
                self._h2d_src = None

    def _ensure_device(self):
        """Make the device copy current (upload the host mirror if newer)."""
        if self._dev_valid:
            return
        self._wait_h2d()
        h = self._host
        nbytes = self._buf.nbytes
        if self._host_pinned:
            j = C.c_void_p()
            check(lib.vkc_h2d(self._gpu._dev.h, self._buf.ptr, h.ctypes.data, nbytes, C.byref(j)))
            self._h2d_job = j.value
        else:
            # pageable source: staged before the call returns
            check(lib.vkc_h2d(self._gpu._dev.h, self._buf.ptr, h.ctypes.data, nbytes, None))
        self._dev_valid = True

    def _ensure_host(self) -> np.ndarray:
        """Make the host mirror current and return it."""
        self._wait_d2h()
        if self._host is None:
            self._host, self._host_pinned = _host_buffer(self.shape, self._dtype)
            self._host_valid = False
        elif self._host.shape != self.shape:
            self._host = self._host.reshape(self.shape)
        if not self._host_valid:
            self._wait_h2d()
            dev = self._gpu._dev
            issued = dev.seq
            if self._size:
                # ordered after every queued op; returns when the copy is done
                check(lib.vkc_d2h(dev.h, self._host.ctypes.data, self._buf.ptr, self._buf.nbytes))
            else:
                dev.synchronize()
            dev.done = max(dev.done, issued)
            self.job = None
            self._keep = []
            self._host_valid = True
        return self._host

    def _dptr(self) -> int:
        """Device pointer for reading (uploads pending host writes first)."""
        self._ensure_device()
        cap = self._gpu._dev.capture
        if cap is not None:
            cap._touch(self, write=False)
        return self._buf.ptr or 0

    def _written(self):
        """Record that an op on the stream (re)wrote this array."""
        self._dev_valid = True
        self._host_valid = False
        self._d2h_fresh = False
        dev = self._gpu._dev
        if dev.capture is not None:
            dev.capture._touch(self, write=True)
            self.job = None
            return
        self.job = dev.issued()

    # -- host access
    @property
    def buffer(self) -> _BufferInfo:
        return _BufferInfo(self)

    @property
    def array(self) -> np.ndarray:
        """Writable host view.  Any access counts as a possible write: the
        host copy is uploaded again before the next op."""
        h = self._ensure_host()
        self._wait_h2d()
        self._dev_valid = False
        return h

    def _info(self):
        return self

    def __getitem__(self, key: KeyType) -> ValueType:
        return self._ensure_host()[key]

    def __setitem__(self, key: KeyType, value: ValueType):
        if self._is_full(key) and np.ndim(value) == 0:
            # whole-array fill: done on the device, no host round trip
            self._ensure_device_for_overwrite()
            if self._dtype == np.float32:
                check(lib.vkc_fill_f32(self._gpu._dev.h, self._buf.ptr or 0, self._size, float(value)))
            else:
                check(lib.vkc_fill_u32(self._gpu._dev.h, self._buf.ptr or 0, self._size, int(value) & 0xFFFFFFFF))
            self._written()
            return
        if (self._is_full(key) and isinstance(value, np.ndarray) and value.shape == self.shape and self._size
                and self._gpu._dev.capture is None):
            # whole-array overwrite from host memory: one copy on the device's
            # stream, after the ops queued on the array -- no read-back of the
            # old contents, no pass through the host mirror (a pinned source is
            # read asynchronously and kept alive until its copy is done)
            src = np.ascontiguousarray(value, dtype=self._dtype)
            self._wait_d2h()   # a read-back in flight still reads the buffer
            self._wait_h2d()   # and an upload in flight still reads its source
            self._ensure_device_for_overwrite()
            dev = self._gpu._dev
            if _is_pinned(src):
                j = C.c_void_p()
                check(lib.vkc_h2d(dev.h, self._buf.ptr, src.ctypes.data, self._buf.nbytes, C.byref(j)))
                self._h2d_job, self._h2d_src = j.value, src
            else:
                check(lib.vkc_h2d(dev.h, self._buf.ptr, src.ctypes.data, self._buf.nbytes, None))
            self._written()
            return
        h = self._ensure_host()
        self._wait_h2d()
        h[key] = value
        self._dev_valid = False

    def _ensure_device_for_overwrite(self):
        # The device copy is about to be overwritten completely: a pending
        # upload may still read the mirror, nothing else is needed.
        self._dev_valid = True

    @staticmethod
    def _is_full(key) -> bool:
        if isinstance(key, slice):
            return key == slice(None)
        if key is Ellipsis:
            return True
        return False

    def __repr__(self) -> str:
        return f"<{self.__class__.__name__}(shape={tuple(self.shape)})>"

    def __str__(self) -> str:
        return str(self._ensure_host())

    def __array__(self, dtype=None, copy=None) -> np.ndarray:
        h = self._ensure_host().view()
        h.flags.writeable = False
        if dtype is not None and np.dtype(dtype) != h.dtype:
            return h.astype(dtype)
        if copy:
            return h.copy()
        return h

    def __len__(self):
        return self.shape[0]

    @property
    def size(self) -> int:
        return self._size

    @property
    def ndim(self) -> int:
        return len(self.shape)

    def reshape(self, shape: Iterable[int]):
        """Reshape in place (vkarray.py:607-622); ValueError if sizes differ."""
        shape = tuple(int(s) for s in np.asarray(shape, dtype=np.int64).reshape(-1))
        if shape.count(-1) > 1:
            raise ValueError("can only specify one unknown dimension")
        if -1 in shape:
            known = _prod(s for s in shape if s != -1)
            if known == 0 or self._size % known:
                raise ValueError(f"cannot reshape array of size {self._size} into shape {shape}")
            shape = tuple(self._size // known if s == -1 else s for s in shape)
        if _prod(shape) != self._size:
            raise ValueError(f"cannot reshape array of size {self._size} into shape {shape}")
        self.shape = shape
        if self._host is not None:
            self._host = self._host.reshape(shape)


class U32Array(_GPUArray):
    """
    GPU array of uint32 for indices and class labels (vkarray.py:191-256).
    No arithmetic.
    """
    _dtype = np.uint32

    def __init__(self, gpu: GPU, *, data: Optional[Iterable[int]] = None,
                 shape: Optional[Iterable[int]] = None):
        super().__init__(gpu)
        if data is not None:
            d = np.ascontiguousarray(np.asarray(data, dtype=np.uint32))
            self._init_storage(d.shape, d)
        else:
            if shape is None:
                raise ValueError("One of `data` or `shape` must be specified.")
            self._init_storage(tuple(np.asarray(shape, dtype=int).reshape(-1)), None)

    def to_onehot(self, num_classes: int) -> "Array":
        """One-hot float rows (vkarray.py:239-253)."""
        return Array(self._gpu, data=np.identity(num_classes, dtype=np.float32)).gather(self, axis=0)


class Shape(U32Array):
    """GPU array of uint32 for a shape (vkarray.py:259-278)."""

    def __init__(self, gpu: GPU, *, data: Optional[Iterable[int]] = None, ndim: Optional[int] = None):
        super().__init__(gpu, data=data, shape=(ndim,) if ndim is not None else None)


def _normalize_axes(axis, ndim) -> List[int]:
    """Distinct axes in [0, ndim), descending; a plain int or a tuple/list of
    ints skips numpy (this runs on every axis reduction)."""
    if isinstance(axis, (int, np.integer)):
        axes = (int(axis),)
    elif isinstance(axis, (tuple, list)) and all(isinstance(a, (int, np.integer)) for a in axis):
        axes = tuple(int(a) for a in axis)
    else:
        axes = tuple(int(a) for a in np.asarray(axis, dtype=np.int64).reshape(-1))
    out = set()
    for a in axes:
        if a < -ndim or a >= ndim:
            raise ValueError(f"axis {a} is out of bounds for array of dimension {ndim}")
        out.add(a % ndim)
    return sorted(out, reverse=True)


class Array(_GPUArray):
    """GPU array of float32 (vkarray.py:281-1521)."""

    def __init__(self, gpu: GPU, *, data=None, shape: Optional[Iterable[int]] = None):
        super().__init__(gpu)
        if data is not None:
            d = np.ascontiguousarray(np.asarray(data, dtype=np.float32))
            self._init_storage(d.shape, d)
        elif shape is not None:
            if type(shape) is tuple and all(type(v) is int for v in shape):
                self._init_storage(shape, None)  # the common internal case, without numpy
            else:
                self._init_storage(tuple(int(v) for v in np.asarray(shape, dtype=int).reshape(-1)), None)
        else:
            raise ValueError("`data` or `shape` must not be `None`.")

    @property
    def _h(self):
        return self._gpu._dev.h

    def _new(self, shape) -> "Array":
        return Array(self._gpu, shape=shape)

    def _check_shape(self, other):
        if tuple(self.shape) != tuple(other.shape):
            raise ValueError(f"Incompatible shapes: {self.shape} vs {other.shape}")

    # ------------------------------------------------------------ binary ops
    def _op(self, other, op: int) -> "Array":
        if not isinstance(other, Array):
            ret = self._new(self.shape)
            check(lib.vkc_binary_scalar(self._h, op, self._dptr(), float(other), ret._buf.ptr or 0, self._size))
            ret._written()
            return ret
        if tuple(self.shape) == tuple(other.shape):
            ret = self._new(self.shape)
            check(lib.vkc_binary(self._h, op, self._dptr(), other._dptr(), ret._buf.ptr or 0, self._size))
            ret._written()
            return ret
        shape, sa, sb, sc, nd = _bcast_plan(tuple(self.shape), tuple(other.shape))
        ret = self._new(shape)
        check(lib.vkc_broadcast_binary(self._h, op, self._dptr(), sa, other._dptr(), sb, ret._buf.ptr or 0, sc, nd))
        ret._written()
        return ret

    def _iop(self, other, op: int) -> "Array":
        if not isinstance(other, Array):
            check(lib.vkc_binary_scalar(self._h, op, self._dptr(), float(other), self._buf.ptr or 0, self._size))
        elif tuple(self.shape) == tuple(other.shape):
            check(lib.vkc_binary(self._h, op, self._dptr(), other._dptr(), self._buf.ptr or 0, self._size))
        else:
            shape = tuple(np.broadcast_shapes(self.shape, other.shape))
            if shape != tuple(self.shape):
                raise ValueError(f"Incompatible shape. {shape} vs {self.shape}")
            nd = len(shape)
            check(lib.vkc_broadcast_binary(
                self._h, op, self._dptr(), shape_arg(shape), other._dptr(),
                shape_arg(_pad(other.shape, nd)), self._buf.ptr or 0, shape_arg(shape), nd))
        self._written()
        return self

    def __add__(self, other): return self._op(other, _lib.ADD)
    def __sub__(self, other): return self._op(other, _lib.SUB)
    def __mul__(self, other): return self._op(other, _lib.MUL)
    def __truediv__(self, other): return self._op(other, _lib.DIV)
    def __pow__(self, other): return self._op(other, _lib.POW)
    def __iadd__(self, other): return self._iop(other, _lib.ADD)
    def __isub__(self, other): return self._iop(other, _lib.SUB)
    def __imul__(self, other): return self._iop(other, _lib.MUL)
    def __itruediv__(self, other): return self._iop(other, _lib.DIV)
    def __ipow__(self, other): return self._iop(other, _lib.POW)
    def __radd__(self, other): return self._op(other, _lib.ADD)
    def __rsub__(self, other): return self._op(other, _lib.RSUB)
    def __rmul__(self, other): return self._op(other, _lib.MUL)
    def __rtruediv__(self, other): return self._op(other, _lib.RDIV)
    def __rpow__(self, other): return self._op(other, _lib.RPOW)

    def max(self, other: Union["Array", float], inplace: bool = False) -> "Array":
        """Element-wise max (vkarray.py:624-650)."""
        return self._iop(other, _lib.MAX) if inplace else self._op(other, _lib.MAX)

    def min(self, other: Union["Array", float], inplace: bool = False) -> "Array":
        """Element-wise min (vkarray.py:652-678)."""
        return self._iop(other, _lib.MIN) if inplace else self._op(other, _lib.MIN)

    # ------------------------------------------------------------ unary ops
    def _unary(self, name: str, inplace: bool) -> "Array":
        op = _lib.UNARY[name]
        if inplace:
            check(lib.vkc_unary(self._h, op, self._dptr(), self._buf.ptr or 0, self._size))
            self._written()
            return self
        ret = self._new(self.shape)
        check(lib.vkc_unary(self._h, op, self._dptr(), ret._buf.ptr or 0, self._size))
        ret._written()
        return ret

    def abs(self, inplace: bool = False): return self._unary("abs", inplace)
    def sign(self, inplace: bool = False): return self._unary("sign", inplace)
    def sin(self, inplace: bool = False): return self._unary("sin", inplace)
    def cos(self, inplace: bool = False): return self._unary("cos", inplace)
    def tan(self, inplace: bool = False): return self._unary("tan", inplace)
    def asin(self, inplace: bool = False): return self._unary("asin", inplace)
    def acos(self, inplace: bool = False): return self._unary("acos", inplace)
    def atan(self, inplace: bool = False): return self._unary("atan", inplace)
    def sinh(self, inplace: bool = False): return self._unary("sinh", inplace)
    def cosh(self, inplace: bool = False): return self._unary("cosh", inplace)
    def tanh(self, inplace: bool = False): return self._unary("tanh", inplace)
    def asinh(self, inplace: bool = False): return self._unary("asinh", inplace)
    def acosh(self, inplace: bool = False): return self._unary("acosh", inplace)
    def atanh(self, inplace: bool = False): return self._unary("atanh", inplace)
    def exp(self, inplace: bool = False): return self._unary("exp", inplace)
    def log(self, inplace: bool = False): return self._unary("log", inplace)
    def exp2(self, inplace: bool = False): return self._unary("exp2", inplace)
    def log2(self, inplace: bool = False): return self._unary("log2", inplace)
    def sqrt(self, inplace: bool = False): return self._unary("sqrt", inplace)
    def invsqrt(self, inplace: bool = False): return self._unary("invsqrt", inplace)

    # ------------------------------------------------------------ clamp
    def clamp(self, min: Union["Array", float], max: Union["Array", float], inplace: bool = False) -> "Array":
        """Element-wise clamp (vkarray.py:1110-1191); array bounds broadcast."""
        lo_arr = isinstance(min, Array)
        hi_arr = isinstance(max, Array)
        shapes = [tuple(self.shape)]
        if lo_arr:
            shapes.append(tuple(min.shape))
        if hi_arr:
            shapes.append(tuple(max.shape))
        shape = tuple(np.broadcast_shapes(*shapes))
        if inplace and shape != tuple(self.shape):
            raise ValueError("Incompatible shape")
        same = all(s == shape for s in shapes)
        out = self if inplace else self._new(shape)
        lo_s = 0.0 if lo_arr else float(min)
        hi_s = 0.0 if hi_arr else float(max)
        if same:
            check(lib.vkc_clamp(self._h, self._dptr(), min._dptr() if lo_arr else None,
                                max._dptr() if hi_arr else None, lo_s, hi_s, out._buf.ptr or 0, out._size))
        else:
            nd = len(shape)
            check(lib.vkc_broadcast_clamp(
                self._h, self._dptr(), shape_arg(_pad(self.shape, nd)),
                min._dptr() if lo_arr else None, shape_arg(_pad(min.shape, nd)) if lo_arr else None, lo_s,
                max._dptr() if hi_arr else None, shape_arg(_pad(max.shape, nd)) if hi_arr else None, hi_s,
                out._buf.ptr or 0, shape_arg(shape), nd))
        out._written()
        return out

    # ------------------------------------------------------------ matmul
    def __matmul__(self, other: "Array") -> "Array":
        """Matrix product (vkarray.py:585-605): contracts the last axis of
        ``self`` with the first axis of ``other``."""
        if (len(self.shape) > 3 or len(other.shape) > 3 or len(self.shape) == 0
                or len(other.shape) == 0 or self.shape[-1] != other.shape[0]):
            raise ValueError(f"Incompatible shapes: {self.shape} vs {other.shape}")
        shape = tuple(self.shape)[:-1] + tuple(other.shape)[1:]
        if len(shape) == 0:
            shape = (1,)
        M = _prod(self.shape[:-1])
        K = int(self.shape[-1])
        N = _prod(other.shape[1:])
        ret = self._new(shape)
        prec = _MATMUL_PRECISION[self._gpu.matmul_precision]
        check(lib.vkc_matmul(self._h, prec, self._dptr(), other._dptr(), ret._buf.ptr or 0, M, K, N))
        ret._written()
        return ret

    # ------------------------------------------------------------ reductions
    def _reduce(self, op: int, axis, keepdims: bool, rebroadcast: bool, scale: float = 1.0) -> "Array":
        if self._size == 0:
            raise ValueError("reduction of an empty array")
        if rebroadcast:
            if not isinstance(axis, (int, np.integer)):
                raise ValueError("When `rebroadcast` is specified, `axis` must be `int`")
            a = _normalize_axes(axis, len(self.shape))[0]
            prev = _prod(self.shape[:a])
            n = int(self.shape[a])
            post = _prod(self.shape[a + 1:])
            ret = self._new(self.shape)
            check(lib.vkc_reduce_axis(self._h, op, self._dptr(), prev, n, post, ret._buf.ptr or 0, 1, scale))
            ret._written()
            return ret
        if axis is None:
            ret = self._new((1,))
            check(lib.vkc_reduce_all(self._h, op, self._gpu.reduce_precision, self._dptr(), self._size,
                                     ret._buf.ptr or 0, scale))
            ret._written()
            if keepdims:
                ret.reshape((1,) * len(self.shape))
            return ret
        axes = _normalize_axes(axis, len(self.shape))
        # Merge runs of adjacent axes: [prev, a_i * a_{i+1}, post] is one pass.
        runs = []
        for a in axes:  # descending
            if runs and runs[-1][0] == a + 1:
                runs[-1][0] = a
            else:
                runs.append([a, a])  # [first, last]
        tmp: Array = self
        shape = list(self.shape)
        for i, (first, last) in enumerate(runs):
            prev = _prod(shape[:first])
            n = _prod(shape[first:last + 1])
            post = _prod(shape[last + 1:])
            new_shape = shape[:first] + shape[last + 1:]
            ret = self._new(tuple(new_shape))
            s = scale if i == len(runs) - 1 else 1.0
            check(lib.vkc_reduce_axis(self._h, op, tmp._dptr(), prev, n, post, ret._buf.ptr or 0, 0, s))
            ret._written()
            tmp = ret
            shape = new_shape
        if keepdims:
            ks = list(self.shape)
            for a in axes:
                ks[a] = 1
            tmp.reshape(tuple(ks))
        return tmp

    def sum(self, axis=None, keepdims: bool = False, rebroadcast: bool = False) -> "Array":
        """Sum of elements (vkarray.py:1278-1306)."""
        return self._reduce(_lib.SUM, axis, keepdims, rebroadcast)

    def prod(self, axis=None, keepdims: bool = False, rebroadcast: bool = False) -> "Array":
        """Product of elements (vkarray.py:1308-1336)."""
        return self._reduce(_lib.PROD, axis, keepdims, rebroadcast)

    def maximum(self, axis=None, keepdims: bool = False, rebroadcast: bool = False) -> "Array":
        """Maximum (vkarray.py:1338-1366)."""
        return self._reduce(_lib.MAXIMUM, axis, keepdims, rebroadcast)

    def minimum(self, axis=None, keepdims: bool = False, rebroadcast: bool = False) -> "Array":
        """Minimum (vkarray.py:1368-1396)."""
        return self._reduce(_lib.MINIMUM, axis, keepdims, rebroadcast)

    def _arg(self, op: int, axis, keepdims: bool) -> U32Array:
        if self._size == 0:
            raise ValueError("attempt to get argmax/argmin of an empty sequence")
        if axis is None:
            ret = U32Array(self._gpu, shape=(1,))
            check(lib.vkc_arg_reduce_all(self._h, op, self._dptr(), self._size, ret._buf.ptr or 0))
            ret._written()
            if keepdims:
                ret.reshape((1,) * len(self.shape))
            return ret
        if not isinstance(axis, (int, np.integer)):
            raise ValueError("`axis` must be `int` or `None`")
        a = _normalize_axes(axis, len(self.shape))[0]
        shape = list(self.shape)
        new_shape = shape[:a] + ([1] if keepdims else []) + shape[a + 1:]
        ret = U32Array(self._gpu, shape=tuple(new_shape))
        if ret._size:
            check(lib.vkc_arg_reduce_axis(self._h, op, self._dptr(), _prod(shape[:a]), int(shape[a]),
                                          _prod(shape[a + 1:]), ret._buf.ptr or 0))
            ret._written()
        return ret

    def argmax(self, axis=None, keepdims: bool = False) -> U32Array:
        """Index of the maximum (numpy ``argmax``: first occurrence, NaN
        wins).  ``axis=None`` gives shape ``(1,)`` like the other full
        reductions.  Not in the reference (README.md:73 lists it as
        missing; example/02-nn.py:96 uses numpy on the host)."""
        return self._arg(_lib.ARGMAX, axis, keepdims)

    def argmin(self, axis=None, keepdims: bool = False) -> U32Array:
        """Index of the minimum (numpy ``argmin`` semantics)."""
        return self._arg(_lib.ARGMIN, axis, keepdims)

    def mean(self, axis=None, keepdims: bool = False, rebroadcast: bool = False) -> "Array":
        """Mean (vkarray.py:1398-1432): the sum scaled in the same launch by
        float32(n_after / n_before), or by float32(1 / shape[axis]) when
        ``rebroadcast`` (the reference divides by shape[axis] in a second op)."""
        if rebroadcast:
            if not isinstance(axis, (int, np.integer)):
                raise ValueError("When `rebroadcast` is specified, `axis` must be `int`")
            n = self.shape[_normalize_axes(axis, len(self.shape))[0]]
            return self._reduce(_lib.SUM, axis, keepdims, True, float(np.float32(1.0 / n)))
        if axis is None:
            n_after = 1
        else:
            axes = _normalize_axes(axis, len(self.shape))
            n_after = _prod(s for i, s in enumerate(self.shape) if i not in axes)
        return self._reduce(_lib.SUM, axis, keepdims, False, float(np.float32(n_after / self._size)))

    # ------------------------------------------------------------ data movement
    def broadcast_to(self, shape: Iterable[int]) -> "Array":
        """Broadcast copy (vkarray.py:1434-1474); ValueError if incompatible."""
        shape = tuple(int(s) for s in np.asarray(shape, dtype=int).reshape(-1))
        try:
            b = tuple(np.broadcast_shapes(self.shape, shape))
        except ValueError:
            raise ValueError(f"Cannot broadcast to {shape}")
        if b != shape:
            raise ValueError(f"Cannot broadcast to {shape}")
        ret = self._new(shape)
        nd = len(shape)
        check(lib.vkc_broadcast_to(self._h, self._dptr(), shape_arg(_pad(self.shape, nd)),
                                   ret._buf.ptr or 0, shape_arg(shape), nd))
        ret._written()
        return ret

    def gather(self, indices: U32Array, axis: Optional[int] = None) -> "Array":
        """Gather (vkarray.py:1476-1521).  Flat: shape = indices.shape.
        With ``axis``: shape = indices.shape + shape[:axis] + shape[axis+1:]."""
        n_idx = indices._size
        if axis is None:
            ret = self._new(indices.shape)
            check(lib.vkc_gather(self._h, self._dptr(), self._size, indices._dptr(), n_idx, ret._buf.ptr or 0))
        else:
            a = _normalize_axes(axis, len(self.shape))[0]
            prev_shape = tuple(self.shape[:a])
            post_shape = tuple(self.shape[a + 1:])
            ret = self._new(tuple(indices.shape) + prev_shape + post_shape)
            check(lib.vkc_gather_axis(self._h, self._dptr(), _prod(prev_shape), int(self.shape[a]),
                                      _prod(post_shape), indices._dptr(), n_idx, ret._buf.ptr or 0))
        ret._written()
        return ret


def matmul(a: Array, b: Array, precision: Optional[str] = None) -> Array:
    """``a @ b`` with an explicit arithmetic: "fp32" (SIMT FMA, the drop-in
    default), "bf16" (tensor cores, fp32 accumulate) or "bf16x3" (split
    bf16 on tensor cores: ~fp32 accuracy, relative error ~1e-6..1e-5)."""
    if precision is None:
        return a @ b
    old = a._gpu.matmul_precision
    if precision not in _MATMUL_PRECISION:
        raise ValueError(f"unknown matmul precision {precision!r}")
    a._gpu.matmul_precision = precision
    try:
        return a @ b
    finally:
        a._gpu.matmul_precision = old


def matmul_grouped(a_list: Sequence["Array"], b_list: Sequence["Array"], precision: Optional[str] = None) -> List[Array]:
    """``[a @ b for a, b in zip(a_list, b_list)]`` for 2-D operands of any
    sizes, computed by one grouped launch (per 128 products) instead of one
    launch per product.  ``precision`` as for ``matmul`` (default: the GPU's
    ``matmul_precision``).  No counterpart in the reference."""
    if len(a_list) != len(b_list):
        raise ValueError("a_list and b_list differ in length")
    if not a_list:
        return []
    gpu = a_list[0]._gpu
    prec = precision or gpu.matmul_precision
    if prec not in _MATMUL_PRECISION:
        raise ValueError(f"unknown matmul precision {prec!r}")
    probs, outs = [], []
    for a, b in zip(a_list, b_list):
        if len(a.shape) != 2 or len(b.shape) != 2 or a.shape[1] != b.shape[0]:
            raise ValueError(f"Incompatible shapes for grouped matmul: {a.shape} @ {b.shape}")
        m, k = a.shape
        n = b.shape[1]
        c = Array(gpu, shape=(m, n))
        outs.append(c)
        probs.append(_lib.GemmProblem(ta=0, tb=0, m=m, n=n, k=k, alpha=1.0, beta=0.0, a=a._dptr(), lda=k,
                                      b=b._dptr(), ldb=n, c=c._buf.ptr or 0, ldc=n, bias=None,
                                      act=_lib.ACT_NONE, relu_mask=None))
    arr = (_lib.GemmProblem * len(probs))(*probs)
    check(lib.vkc_gemm_grouped(gpu._dev.h, _MATMUL_PRECISION[prec], arr, len(probs)))
    for c in outs:
        c._written()
    return outs


@functools.lru_cache(maxsize=256)
def _bcast_plan(a_shape: tuple, b_shape: tuple):
    """Result shape and the C shape arguments of a broadcast binary op (the
    ctypes arrays are read-only for the library, so one set per pair of
    shapes serves every call)."""
    shape = tuple(int(v) for v in np.broadcast_shapes(a_shape, b_shape))
    nd = len(shape)
    return shape, shape_arg(_pad(a_shape, nd)), shape_arg(_pad(b_shape, nd)), shape_arg(shape), nd


def _pad(shape, nd) -> tuple:
    shape = tuple(int(s) for s in shape)
    return (1,) * (nd - len(shape)) + shape


def zeros(gpu: GPU, shape: Iterable[int]) -> Array:
    """Zero-initialised Array (vkarray.py:1524-1542), filled on the device."""
    z = Array(gpu, shape=shape)
    z[:] = 0.0
    return z
