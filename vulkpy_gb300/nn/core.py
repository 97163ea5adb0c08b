"""
Abstract base classes of the nn library (names and contracts of
vulkpy/nn/core.py:22-337).
"""
from __future__ import annotations

from typing import Iterable

from ..vkarray import GPU, Array

__all__ = ["OptimizerState", "Optimizer", "Regularizer", "Loss", "Module"]


class OptimizerState:
    """Per-parameter mutable optimizer values (core.py:22-63).

    ``grad2diff(grad)`` returns the update difference (``v += diff``);
    ``apply(value, grad)`` performs ``value += grad2diff(grad)`` in place
    (a single fused kernel in the built-in optimizers)."""

    def grad2diff(self, grad: Array) -> Array:
        raise NotImplementedError

    def apply(self, value: Array, grad: Array):
        value += self.grad2diff(grad)


class Optimizer:
    """Optimizer: holds global hyper-parameters, creates states (core.py:66-113)."""

    def init_state(self, shape: Iterable[int]) -> OptimizerState:
        raise NotImplementedError


class Loss:
    """Loss: ``__call__(x, y)`` computes it, ``grad()`` returns dL/dx (core.py:116-168)."""

    def __call__(self, x: Array, y: Array) -> Array:
        raise NotImplementedError

    def grad(self) -> Array:
        raise NotImplementedError


class Regularizer:
    """Regularizer: ``loss(param)`` and ``grad(param)`` (core.py:171-221)."""

    def loss(self, param: Array) -> Array:
        raise NotImplementedError

    def grad(self, param: Array) -> Array:
        raise NotImplementedError


class Module:
    """Layer base class (core.py:224-337).

    ``__call__`` requires an input of at least two dimensions and stores the
    input and output for ``backward``."""

    def __call__(self, x: Array) -> Array:
        if len(x.shape) < 2:
            raise ValueError("Input must have at least 2-dimensions.")
        self._x = x
        self._y = self.forward(x)
        return self._y

    def forward(self, x: Array) -> Array:
        raise NotImplementedError

    def backward(self, dy: Array) -> Array:
        raise NotImplementedError

    def zero_grad(self):
        pass

    def update(self):
        pass
