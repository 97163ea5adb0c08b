"""
Losses (vulkpy/nn/losses.py:40-458).

Cross entropy (optionally fused with the softmax) computes each row's loss
in one kernel; the batch reduction (mean or sum over axis 0) and the
backward scaling 1/batch follow the reference's ReduceLoss (losses.py:40-92).
"""
from __future__ import annotations

from typing import Callable, Iterable, Literal, Optional, Tuple, cast

import numpy as np

from ..vkarray import Array
from .._lib import lib, check
from .core import Loss
from .layers import Softmax

__all__ = ["CrossEntropyLoss", "SoftmaxCrossEntropyLoss", "MSELoss", "HuberLoss", "MixLoss"]

F = Callable[[Array], Array]


class ReduceLoss(Loss):
    def __init__(self, reduce: Literal["mean", "sum"] = "mean"):
        tmp: Tuple[F, Optional[F]] = {
            "mean": (lambda _L: _L.mean(axis=0), lambda _dx: 1 / _dx.shape[0]),
            "sum": (lambda _L: _L.sum(axis=0), None),
        }[reduce]
        self.reduce, self.scale_backward = tmp

    def __call__(self, x: Array, y: Array) -> Array:
        self._x = x
        self._y = y
        L = self.forward(x, y)
        return self.reduce(L)

    def grad(self) -> Array:
        dx = self.backward()
        if self.scale_backward is not None:
            dx *= self.scale_backward(dx)
        return dx

    def forward(self, x: Array, y: Array) -> Array:
        raise NotImplementedError

    def backward(self) -> Array:
        raise NotImplementedError


def _ce_rows(x: Array, y: Array, softmax: bool, p_out: Optional[Array]) -> Array:
    rows = Array(x._gpu, shape=(x.shape[0],))
    check(lib.vkc_cross_entropy(x._h, x._dptr(), y._dptr(), rows._buf.ptr or 0,
                                p_out._buf.ptr if p_out is not None else None, x.shape[0], x.shape[1],
                                1 if softmax else 0))
    rows._written()
    if p_out is not None:
        p_out._written()
    return rows


class CrossEntropyLoss(ReduceLoss):
    """L = sum_c -y log(x + 1e-8); dL/dx = -y / (x + 1e-8) (losses.py:95-176)."""

    def forward(self, x: Array, y: Array) -> Array:
        if len(x.shape) == 2:
            return _ce_rows(x, y, False, None)
        L = x + 1e-8
        L.log(inplace=True)
        L *= y
        L *= -1.0
        return L.sum(axis=1)

    def backward(self) -> Array:
        dx = self._y / (self._x + 1e-8)
        dx *= -1.0
        return dx


class SoftmaxCrossEntropyLoss(CrossEntropyLoss):
    """Cross entropy of softmax(x); dL/dx = softmax(x) - y (losses.py:179-249).

    For a 2-D batch of up to 2048 rows the loss step runs as two kernels:
    row losses, softmax and the gradient that ``grad()`` then returns in the
    first, their batch mean (or sum) in the second, with the same float32
    results as the separate row-loss, reduction and gradient kernels."""

    _FUSED_MAX_ROWS = 2048

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self._sm = Softmax()
        self._dx: Optional[Array] = None

    def __call__(self, x: Array, y: Array) -> Array:
        self._dx = None
        if (len(x.shape) == 2 and tuple(y.shape) == tuple(x.shape)
                and 1 <= x.shape[0] <= self._FUSED_MAX_ROWS and x.shape[1] >= 1):
            self._x = x
            self._y = y
            rows = x.shape[0]
            gpu = x._gpu
            p = Array(gpu, shape=x.shape)
            dx = Array(gpu, shape=x.shape)
            loss = Array(gpu, shape=())
            mean = self.scale_backward is not None
            # ReduceLoss: mean(axis=0) scales by float32(1 / rows) in the
            # reduction; grad() by the Python float 1 / rows
            lscale = float(np.float32(1.0 / rows)) if mean else 1.0
            gscale = self.scale_backward(dx) if mean else 1.0
            check(lib.vkc_softmax_ce_fused(x._h, x._dptr(), y._dptr(), p._buf.ptr or 0, dx._buf.ptr or 0,
                                           loss._buf.ptr or 0, rows, x.shape[1], lscale, float(gscale)))
            for a in (p, dx, loss):
                a._written()
            self._sm._x = x
            self._sm._y = p
            self._dx = dx
            return loss
        return super().__call__(x, y)

    def forward(self, x: Array, y: Array) -> Array:
        if len(x.shape) == 2:
            p = Array(x._gpu, shape=x.shape)
            rows = _ce_rows(x, y, True, p)
            self._sm._x = x
            self._sm._y = p
            return rows
        return super().forward(self._sm(x), y)

    def backward(self) -> Array:
        return cast(Array, self._sm._y) - self._y

    def grad(self) -> Array:
        """(softmax(x) - y) * scale in one kernel: the same two float32 ops
        as backward() followed by ReduceLoss's 1/batch scaling (already
        computed by the fused loss step when that ran)."""
        if self._dx is not None:
            return self._dx
        p = cast(Array, self._sm._y)
        scale = 1.0 if self.scale_backward is None else self.scale_backward(p)
        dx = Array(p._gpu, shape=p.shape)
        check(lib.vkc_softmax_ce_backward(p._h, p._dptr(), self._y._dptr(), dx._buf.ptr or 0, dx._size,
                                          float(scale)))
        dx._written()
        return dx


class MSELoss(ReduceLoss):
    """L = sum (y - x)^2; dL/dx = 2 (x - y) (losses.py:252-320)."""

    def forward(self, x: Array, y: Array) -> Array:
        L = y - x
        L **= 2.0
        return L.sum(axis=1)

    def backward(self) -> Array:
        dx = self._x - self._y
        dx *= 2
        return dx


class HuberLoss(ReduceLoss):
    """L = 0.5 min(|d|, d^2) summed; dL/dx = clamp(x - y, -1, 1) (losses.py:323-393)."""

    def forward(self, x: Array, y: Array) -> Array:
        delta = y - x
        delta.abs(inplace=True)
        delta.min(delta ** 2.0, inplace=True)
        delta *= 0.5
        return delta.sum(axis=1)

    def backward(self) -> Array:
        delta = self._x - self._y
        delta.clamp(-1.0, 1.0, inplace=True)
        return delta


class MixLoss(Loss):
    """Weighted sum of losses (losses.py:396-458)."""

    def __init__(self, losses: Iterable[Tuple[float, Loss]]):
        self.L: Tuple[Tuple[float, Loss], ...] = tuple(losses)
        if len(self.L) < 1:
            raise ValueError("losses should not empty")

    def __call__(self, x: Array, y: Array) -> Array:
        return self._sum(lambda _L: _L(x, y))

    def grad(self) -> Array:
        return self._sum(lambda _L: _L.grad())

    def _sum(self, F: Callable[[Loss], Array]) -> Array:
        coeff, _L = self.L[0]
        s = coeff * F(_L)
        for coeff, _L in self.L[1:]:
            s += coeff * F(_L)
        return s
