"""Regularizers (vulkpy/nn/regularizers.py:23-192)."""
from __future__ import annotations

import logging

from ..vkarray import Array
from .core import Regularizer

__all__ = ["Lasso", "Ridge", "Elastic"]

logger = logging.getLogger("vulkpy_gb300")


class Lasso(Regularizer):
    """L1: loss = coeff * sum|p|, grad = coeff * sign(p)."""

    def __init__(self, coeff: float = 1.0):
        logger.debug(f"Lasso(L1={coeff})")
        self.coeff: float = coeff

    def loss(self, param: Array) -> Array:
        L = param.abs().sum()
        L *= self.coeff
        return L

    def grad(self, param: Array) -> Array:
        return self.coeff * param.sign()


class Ridge(Regularizer):
    """L2: loss = coeff * sum p^2, grad = 2 coeff p."""

    def __init__(self, coeff: float = 1.0):
        logger.debug(f"Ridge(L2={coeff})")
        self.coeff: float = coeff

    def loss(self, param: Array) -> Array:
        L = (param ** 2).sum()
        L *= self.coeff
        return L

    def grad(self, param: Array) -> Array:
        return 2 * self.coeff * param


class Elastic(Regularizer):
    """L1 + L2."""

    def __init__(self, L1: float = 1.0, L2: float = 1.0):
        self.L1 = Lasso(L1)
        self.L2 = Ridge(L2)

    def loss(self, param: Array) -> Array:
        return self.L1.loss(param) + self.L2.loss(param)

    def grad(self, param: Array) -> Array:
        return self.L1.grad(param) + self.L2.grad(param)
