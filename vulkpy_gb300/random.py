"""
Random module (drop-in for vulkpy.random, vulkpy/random.py:1-312).

xoshiro128++ with vulkpy's seeding and chunked stream layout, bit-exact on
the raw uint32 stream.  Seeding runs on the GPU; each ``random``/``randint``/
``normal``/``randrange`` call is a single kernel launch (the reference
submits one job per chunk of ``size`` outputs, _vkarray.cc:697-717).

>>> import vulkpy_gb300 as vk
>>> gpu = vk.GPU()
>>> r = vk.random.Xoshiro128pp(gpu, seed=0)
>>> u = r.random(shape=(3,))
>>> z = r.normal(shape=(3,))
"""
from __future__ import annotations

import secrets
from typing import Iterable, Optional

import numpy as np

from . import vkarray as vk
from ._lib import lib, check

__all__ = ["Xoshiro128pp"]


class PRNG(vk.Resource):
    """Base class (random.py:40-190)."""

    _2p32 = int(2 ** 32)

    def __init__(self, gpu: vk.GPU):
        self._gpu = gpu

    def random(self, *, shape: Optional[Iterable[int]] = None, buffer: Optional[vk.Array] = None) -> vk.Array:
        raise NotImplementedError

    def randint(self, *, shape: Optional[Iterable[int]] = None,
                buffer: Optional[vk.U32Array] = None) -> vk.U32Array:
        raise NotImplementedError

    def normal(self, *, shape: Optional[Iterable[int]] = None, buffer: Optional[vk.Array] = None,
               mean: float = 0.0, stddev: float = 1.0) -> vk.Array:
        raise NotImplementedError

    def randrange(self, *, shape: Optional[Iterable[int]] = None, buffer: Optional[vk.U32Array] = None,
                  low: int = 0, high: int = int(2 ** 32)) -> vk.U32Array:
        raise NotImplementedError

    def wait(self):
        pass


def _target(gpu, shape, buffer, cls):
    if buffer is None:
        if shape is None:
            raise ValueError("One of `shape` and `buffer` must be specified.")
        return cls(gpu, shape=shape)
    # The whole buffer is overwritten: pending host writes are irrelevant.
    buffer._dev_valid = True
    return buffer


class Xoshiro128pp(PRNG):
    """
    xoshiro128++ pseudo random number generator (random.py:192-312).

    ``size`` independent states are seeded from ``seed`` exactly like
    vulkpy (splitmix64 chain, then vulkpy's jump between states) and
    generate numbers in parallel.  Output ``k`` of a call comes from state
    ``k % size`` and the states advance in place between calls.
    """

    def __init__(self, gpu: vk.GPU, size: int = 64, *, seed: Optional[int] = None):
        super().__init__(gpu)
        size = int(size)
        if size <= 0 or size >= 2 ** 32:
            raise ValueError(f"size must be in [1, 2^32), got {size}")
        self.size = size
        if seed is None:
            # the reference draws std::random_device{}(), 32 bits
            seed = secrets.randbits(32)
        seed = int(seed)
        if seed < 0 or seed >= 2 ** 64:
            raise ValueError("seed must be a non-negative 64-bit integer")
        self._state = vk.U32Array(gpu, shape=(4 * size,))
        check(lib.vkc_xoshiro_seed(gpu._dev.h, seed, size, self._state._buf.ptr))
        self._state._written()

    def state(self) -> np.ndarray:
        """Current states as a (size, 4) uint32 array (host copy)."""
        return np.array(self._state, copy=True).reshape(self.size, 4)

    def random(self, *, shape: Optional[Iterable[int]] = None, buffer: Optional[vk.Array] = None) -> vk.Array:
        """[0, 1) floats from the top 23 bits of each output."""
        buf = _target(self._gpu, shape, buffer, vk.Array)
        check(lib.vkc_xoshiro_f32(self._gpu._dev.h, self._state._buf.ptr, self.size, buf._buf.ptr or 0, buf._size))
        buf._written()
        self._state._written()
        return buf

    def randint(self, *, shape: Optional[Iterable[int]] = None,
                buffer: Optional[vk.U32Array] = None) -> vk.U32Array:
        """Raw uint32 outputs in [0, 2^32)."""
        buf = _target(self._gpu, shape, buffer, vk.U32Array)
        check(lib.vkc_xoshiro_u32(self._gpu._dev.h, self._state._buf.ptr, self.size, buf._buf.ptr or 0, buf._size))
        buf._written()
        self._state._written()
        return buf

    def normal(self, *, shape: Optional[Iterable[int]] = None, buffer: Optional[vk.Array] = None,
               mean: float = 0.0, stddev: float = 1.0) -> vk.Array:
        """Gaussian numbers by Box-Muller on pairs of the uniform stream
        (random.py:60-124).  An odd count draws one extra uniform, like the
        reference; unlike it, the last element is written too."""
        buf = _target(self._gpu, shape, buffer, vk.Array)
        check(lib.vkc_xoshiro_normal(self._gpu._dev.h, self._state._buf.ptr, self.size, buf._buf.ptr or 0,
                                     buf._size, float(mean), float(stddev)))
        buf._written()
        self._state._written()
        return buf

    def randrange(self, *, shape: Optional[Iterable[int]] = None, buffer: Optional[vk.U32Array] = None,
                  low: int = 0, high: int = int(2 ** 32)) -> vk.U32Array:
        """[low, high) integers as ``low + uint(float(high - low) * u)``
        (random.py:126-186, prng_randrange.comp:20-27)."""
        if low < 0:
            raise ValueError(f"`low` must be non negative integer, but {low}")
        if high > self._2p32:
            raise ValueError(f"`high` must not be greater than 2^32, but {high}")
        if low >= high:
            raise ValueError(f"`low` must be smaller than `high`, but {low}, {high}")
        if low == 0 and high == self._2p32:
            return self.randint(shape=shape, buffer=buffer)
        buf = _target(self._gpu, shape, buffer, vk.U32Array)
        check(lib.vkc_xoshiro_randrange(self._gpu._dev.h, self._state._buf.ptr, self.size, buf._buf.ptr or 0,
                                        buf._size, int(low), int(high) - 1))
        buf._written()
        self._state._written()
        return buf

    def permutation(self, n: int) -> vk.U32Array:
        """A pseudo-random permutation of ``0..n-1`` computed on the device.

        The reference shuffles on the host (example/02-nn.py:82).  Four
        uint32 are drawn from this generator as keys of a Feistel-network
        bijection, so a seeded generator gives a reproducible order; each
        index is computed independently (one launch, no sort)."""
        n = int(n)
        if n < 0 or n >= self._2p32:
            raise ValueError(f"n must be in [0, 2^32), got {n}")
        buf = vk.U32Array(self._gpu, shape=(n,))
        check(lib.vkc_xoshiro_permutation(self._gpu._dev.h, self._state._buf.ptr, self.size,
                                          buf._buf.ptr or 0, n))
        buf._written()
        if n:
            self._state._written()
        return buf

    def shuffle(self, x: vk.Array) -> None:
        """Shuffle ``x`` in place along its first axis (numpy
        ``Generator.shuffle`` semantics) with ``permutation(len(x))``."""
        if len(x.shape) == 0 or x.shape[0] <= 1:
            return
        y = x.gather(self.permutation(x.shape[0]), axis=0)
        src = y._dptr()
        x._ensure_device_for_overwrite()
        check(lib.vkc_copy(self._gpu._dev.h, x._buf.ptr, src, x._size * 4))
        x._written()
