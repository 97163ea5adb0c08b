"""Parameter (vulkpy/nn/parameters.py:14-116)."""
from __future__ import annotations

from typing import Callable, Iterable, Optional

from ..vkarray import GPU, Array, zeros
from .core import Optimizer, OptimizerState, Regularizer
from .optimizers import Adam

__all__ = ["Parameter"]


class Parameter:
    """Value, accumulated gradient, optimizer state and optional regularizer."""

    def __init__(self, gpu: GPU, shape: Iterable[int], trainable: bool = True, opt: Optional[Optimizer] = None,
                 initializer: Optional[Callable[[GPU, Iterable[int]], Array]] = None,
                 regularizer: Optional[Regularizer] = None):
        if initializer is None:
            initializer = zeros
        self.value: Array = initializer(gpu, shape)
        self.grad: Optional[Array] = None
        self.opt_state: Optional[OptimizerState] = None
        if trainable:
            self.grad = zeros(gpu, shape=shape)
            if opt is None:
                opt = Adam(gpu)
            self.opt_state = opt.init_state(shape)
        self.R: Optional[Regularizer] = regularizer

    def is_trainable(self) -> bool:
        return self.grad is not None

    def add_grad(self, grad: Array):
        if self.grad is not None:
            self.grad += grad

    def zero_grad(self):
        if self.grad is not None:
            self.grad[:] = 0.0

    def update(self):
        if self.grad is not None:
            self.opt_state.apply(self.value, self.grad)

    def regular_loss(self) -> Array:
        if self.R is not None:
            return self.R.loss(self.value)
        return zeros(self.value._gpu, shape=(1,))

    def regular_grad(self):
        if self.R is not None:
            self.add_grad(self.R.grad(self.value))
