"""
CUDA-graph capture of a sequence of array ops (no counterpart in vulkpy,
which submits every op as its own Vulkan job, _vkarray.cc:403-438).

>>> g = vk.graph.Graph(gpu)
>>> with g:                       # ops are recorded, not run
...     y = (x * 2.0).exp()
>>> g.launch()                    # runs the recorded ops; y holds the result
>>> g.launch(flush=[x])           # after host writes to x, upload them first

Rules while capturing: no host reads or waits, no new arrays from host data
(``Array(data=...)``); arrays created inside the capture keep their device
addresses across launches and are rewritten by every launch; arrays read or
written by the captured ops are kept alive by the graph.
"""
from __future__ import annotations

import ctypes as C
import weakref
from typing import Iterable

from ._lib import lib, check

__all__ = ["Graph"]


class Graph:
    def __init__(self, gpu):
        self._gpu = gpu
        self._dev = gpu._dev
        self._h = None
        self._allocated = set()     # graph allocations still live
        self._deferred = []         # frees of older buffers requested during capture
        self._keep = {}             # external arrays used by the captured ops
        self._written = {}          # weakrefs to arrays the captured ops write
        self._launched = False

    def _touch(self, arr, write: bool):
        key = id(arr)
        if arr._buf is not None and arr._buf.graph is not self:
            self._keep.setdefault(key, arr)
        if write:
            # ids of arrays freed during the capture are reused by later
            # objects: replace an entry that no longer names this array
            r = self._written.get(key)
            if r is None or r() is not arr:
                self._written[key] = weakref.ref(arr)
            if arr._buf is not None and arr._buf.graph is self:
                arr._graph = self   # keep the graph alive while this array lives

    def __enter__(self):
        if self._h is not None:
            raise RuntimeError("graph already captured")
        if self._dev.capture is not None:
            raise RuntimeError("another graph is being captured on this device")
        check(lib.vkc_graph_begin(self._dev.h))
        self._dev.capture = self
        return self

    def __exit__(self, exc_type, exc, tb):
        h = C.c_void_p()
        st = lib.vkc_graph_end(self._dev.h, C.byref(h))
        self._dev.capture = None
        for p in self._deferred:
            lib.vkc_free(self._dev.h, p)
        self._deferred = []
        self._dev.reap()
        if exc_type is not None:
            if h.value:
                lib.vkc_graph_destroy(h)
            return False
        check(st)
        self._h = h
        return False

    def launch(self, flush: Iterable = ()):
        """Run the captured ops once on the device's stream (asynchronous)."""
        if self._h is None:
            raise RuntimeError("graph not captured")
        for a in flush:
            a._ensure_device()
        check(lib.vkc_graph_launch(self._h))
        self._launched = True
        for r in self._written.values():
            a = r()
            if a is not None:
                a._dev_valid = True
                a._host_valid = False
                a.job = self._dev.issued()

    def __del__(self):
        # The garbage collector may run this in the middle of another
        # graph's capture (graphs sit in reference cycles with their arrays),
        # where destroying a graph or freeing its memory would invalidate that
        # capture: the device defers both until no capture or branch is open.
        try:
            # graph allocations exist once the graph has run; the last
            # launch's live ones are released with it
            ptrs = list(self._allocated) if self._launched else []
            self._allocated = set()
            h, self._h = self._h, None
            if h is not None or ptrs:
                self._dev.zombies.append((h, ptrs))
                self._dev.reap()
        except Exception:  # interpreter shutdown
            pass
