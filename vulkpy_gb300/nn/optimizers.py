"""
Optimizers (vulkpy/nn/optimizers.py:24-350).

Each state's ``apply(value, grad)`` is one fused kernel that reproduces the
reference's chain of float32 array ops element by element (same roundings,
no FMA contraction), so parameters match the unfused reference bit for bit.
``grad2diff`` keeps the reference's contract and returns the difference.
"""
from __future__ import annotations

import logging
from typing import Iterable

import numpy as np

from ..vkarray import GPU, Array, U32Array, zeros
from .._lib import lib, check
from .core import Optimizer, OptimizerState

__all__ = ["SGD", "SGDState", "AdaGrad", "AdaGradState", "Adam", "AdamState", "Optimizer", "OptimizerState"]

logger = logging.getLogger("vulkpy_gb300")


class SGDState(OptimizerState):
    """SGD state (optimizers.py:24-52): diff = -lr * grad."""

    def __init__(self, opt: "SGD"):
        self.opt: SGD = opt

    def grad2diff(self, grad: Array) -> Array:
        return -self.opt.lr * grad

    def apply(self, value: Array, grad: Array):
        check(lib.vkc_sgd_update(value._h, value._dptr(), grad._dptr(), value._size, float(self.opt.lr)))
        value._written()


class SGD(Optimizer):
    """Stochastic gradient descent (optimizers.py:55-96)."""

    def __init__(self, lr: float):
        self.lr: float = lr
        logger.debug("SGD(lr=%f)", self.lr)

    def init_state(self, shape: Iterable[int]) -> SGDState:
        return SGDState(self)


class AdaGradState(OptimizerState):
    """AdaGrad state (optimizers.py:99-139): h += g^2; diff = -lr * g / (sqrt(h) + eps)."""

    def __init__(self, opt: "AdaGrad", shape: Iterable[int], tau: float):
        self.opt: AdaGrad = opt
        self.h: Array = zeros(self.opt.gpu, shape=shape)
        self.h[:] = tau

    def grad2diff(self, grad: Array) -> Array:
        diff = zeros(self.opt.gpu, shape=grad.shape)
        self.apply(diff, grad)
        return diff

    def apply(self, value: Array, grad: Array):
        check(lib.vkc_adagrad_update(value._h, value._dptr(), grad._dptr(), self.h._dptr(), value._size,
                                     float(self.opt.lr), float(self.opt.eps)))
        self.h._written()
        value._written()


class AdaGrad(Optimizer):
    """AdaGrad (optimizers.py:142-197)."""

    def __init__(self, gpu: GPU, *, lr: float = 0.01, tau: float = 0.0, eps: float = 1e-8):
        self.gpu: GPU = gpu
        self.lr: float = lr
        self.tau: float = tau
        self.eps: float = eps
        logger.debug("AdaGrad(lr=%f, tau=%f, eps=%f)", self.lr, self.tau, self.eps)

    def init_state(self, shape: Iterable[int]) -> AdaGradState:
        return AdaGradState(opt=self, shape=shape, tau=self.tau)


class AdamState(OptimizerState):
    """Adam state (optimizers.py:200-253): first/second moments and the
    running powers beta1^t, beta2^t (Python floats, as in the reference)."""

    def __init__(self, opt: "Adam", shape: Iterable[int]):
        self.opt: Adam = opt
        self.m: Array = zeros(self.opt.gpu, shape=shape)
        self.v: Array = zeros(self.opt.gpu, shape=shape)
        self.beta1t: float = 1.0
        self.beta2t: float = 1.0
        # the same running powers on the device (two doubles and the update
        # kernel's completion counter), advanced by the update kernel itself
        # so that a captured training step can be replayed
        self._powers = U32Array(self.opt.gpu, data=np.array([1.0, 1.0, 0.0], dtype=np.float64).view(np.uint32))

    def grad2diff(self, grad: Array) -> Array:
        diff = zeros(self.opt.gpu, shape=grad.shape)
        self.apply(diff, grad)
        return diff

    def apply(self, value: Array, grad: Array):
        self.beta1t *= self.opt.beta1
        self.beta2t *= self.opt.beta2
        check(lib.vkc_adam_update_dev(value._h, value._dptr(), grad._dptr(), self.m._dptr(), self.v._dptr(),
                                      value._size, float(self.opt.lr), float(self.opt.beta1),
                                      float(self.opt.beta2), float(self.opt.eps), self._powers._dptr()))
        self._powers._written()
        self.m._written()
        self.v._written()
        value._written()


class Adam(Optimizer):
    """Adam (optimizers.py:256-350)."""

    def __init__(self, gpu: GPU, *, lr: float = 0.001, beta1: float = 0.9, beta2: float = 0.999,
                 eps: float = 1e-8):
        self.gpu: GPU = gpu
        self.lr: float = lr
        self.beta1: float = beta1
        self.beta2: float = beta2
        self.eps: float = eps
        logger.debug("Adam(lr=%f, beta1=%f, beta2=%f, eps=%f)", self.lr, self.beta1, self.beta2, self.eps)

    def init_state(self, shape: Iterable[int]) -> AdamState:
        return AdamState(opt=self, shape=shape)
