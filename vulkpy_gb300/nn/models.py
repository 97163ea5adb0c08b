"""Sequential model (vulkpy/nn/models.py:15-105)."""
from __future__ import annotations

from typing import Iterable, Optional, Tuple, Union

from ..vkarray import Array
from .core import Module, Loss

__all__ = ["Sequence"]


class Sequence:
    """Layers applied in order, trained against one loss.

    Like the reference, parameter regularizers are not applied by ``train``
    (vulkpy's Sequence never calls ``regular_grad``); pass
    ``apply_regularizers=True`` to add their gradients before the update."""

    def __init__(self, layers: Iterable[Module], loss: Loss, *, apply_regularizers: bool = False):
        self.L: Tuple[Module, ...] = tuple(layers)
        self.loss: Loss = loss
        self.apply_regularizers = apply_regularizers

    def _forward(self, x: Array) -> Array:
        for _L in self.L:
            x = _L(x)
        return x

    def _backward(self):
        dx = self.loss.grad()
        for _L in self.L[::-1]:
            dx = _L.backward(dx)

    def _zero_grad(self):
        for _L in self.L:
            _L.zero_grad()

    def _update(self):
        for _L in self.L:
            if self.apply_regularizers:
                for p in (getattr(_L, "w", None), getattr(_L, "b", None)):
                    if p is not None:
                        p.regular_grad()
            _L.update()

    def train(self, x: Array, y: Array) -> Tuple[Array, Array]:
        """One step: forward, loss, zero_grad, backward, update (models.py:55-78)."""
        _y = self._forward(x)
        _loss = self.loss(_y, y)
        self._zero_grad()
        self._backward()
        self._update()
        return (_y, _loss)

    def predict(self, x: Array, y: Optional[Array] = None) -> Union[Array, Tuple[Array, Array]]:
        """Forward only; with ``y`` also the loss (models.py:80-105)."""
        _y = self._forward(x)
        if y is None:
            return _y
        _loss = self.loss(_y, y)
        return (_y, _loss)
