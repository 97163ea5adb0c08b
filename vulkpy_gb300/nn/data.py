"""
Device-side minibatching for training loops.

The reference's training example shuffles an index array on the host and
uploads every batch (example/02-nn.py:77-91, "TODO: Implement GPU
shuffle()").  Here the data set stays in device memory: the rows are
permuted on the device by ``Xoshiro128pp.permutation`` (one launch) and each
batch is one row gather, so an epoch does no host-to-device copies and can
be captured in a CUDA graph whole (the generator state advances on the
device, so every replay draws a new order).

>>> import numpy as np, vulkpy_gb300 as vk
>>> from vulkpy_gb300 import nn
>>> gpu = vk.GPU()
>>> X = vk.Array(gpu, data=np.zeros((120, 4)))
>>> Y = vk.Array(gpu, data=np.zeros((120, 3)))
>>> rng = vk.random.Xoshiro128pp(gpu, seed=0)
>>> for x, y in nn.minibatches(X, Y, 32, rng=rng):
...     pass
"""
from __future__ import annotations

from typing import Dict, Iterator, List, Optional, Tuple

import numpy as np

from ..vkarray import Array, U32Array

__all__ = ["minibatches"]

# Row-range index arrays, built once per (device, rows, batch size) so that a
# later epoch (or a graph capture of one) uploads nothing.
_RANGES: Dict[Tuple[int, int, int, bool], List[U32Array]] = {}


def _ranges(gpu, n: int, batch_size: int, drop_last: bool) -> List[U32Array]:
    key = (id(gpu._dev), n, batch_size, drop_last)
    r = _RANGES.get(key)
    if r is None:
        r = []
        for start in range(0, n, batch_size):
            stop = min(start + batch_size, n)
            if drop_last and stop - start < batch_size:
                break
            r.append(U32Array(gpu, data=np.arange(start, stop, dtype=np.uint32)))
        _RANGES[key] = r
    return r


def minibatches(x: Array, y: Optional[Array], batch_size: int, *, rng=None,
                drop_last: bool = False) -> Iterator[Tuple[Array, Optional[Array]]]:
    """Yield ``(x_batch, y_batch)`` pairs of consecutive rows.

    With ``rng`` (a ``Xoshiro128pp``) the rows of ``x`` and ``y`` are first
    permuted together by ``rng.permutation(len(x))``; without it the order is
    kept.  The last batch is smaller when ``batch_size`` does not divide the
    row count, unless ``drop_last``.  The first call for a given row count
    and batch size uploads the row-range tables, so make it before any graph
    capture that uses them."""
    n = int(x.shape[0])
    if y is not None and int(y.shape[0]) != n:
        raise ValueError(f"x and y have different row counts: {n} vs {y.shape[0]}")
    if batch_size <= 0:
        raise ValueError("batch_size must be positive")
    gpu = x._gpu
    ranges = _ranges(gpu, n, int(batch_size), bool(drop_last))
    if rng is not None and n > 1:
        perm = rng.permutation(n)
        x = x.gather(perm, axis=0)
        y = y.gather(perm, axis=0) if y is not None else None
    for idx in ranges:
        yield x.gather(idx, axis=0), (y.gather(idx, axis=0) if y is not None else None)
