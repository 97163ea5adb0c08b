"""
Layers (vulkpy/nn/layers.py:18-323).

Dense runs one fused GEMM+bias kernel forward and two GEMMs plus a column
sum backward, accumulating straight into the parameter gradients (the
reference builds a (batch, out, in) product and sums it, layers.py:131-135);
``backward_act`` also takes the following activation's backward into the
column-sum kernel.
Softmax forward is one fused kernel per row.  The backward formulas are the
reference's, including Softmax's diagonal-only gradient dy*y*(1-y)
(layers.py:302-323), kept for drop-in parity.
"""
from __future__ import annotations

from typing import Callable, Iterable, Optional

from ..vkarray import GPU, Array
from .._lib import lib, check
from .. import _lib
from .core import Module, Optimizer, Regularizer
from .parameters import Parameter
from .initializers import HeNormal

__all__ = ["Dense", "ReLU", "Sigmoid", "Softmax"]

_PREC = {"fp32": _lib.MM_FP32, "bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}


class Dense(Module):
    """Fully connected layer y = x W^T + b, W of shape (output_dim, input_dim)."""

    def __init__(self, gpu: GPU, input_dim: int, output_dim: int, *,
                 w_init: Optional[Callable[[GPU, Iterable[int]], Array]] = None,
                 b_init: Optional[Callable[[GPU, Iterable[int]], Array]] = None,
                 w_opt: Optional[Optimizer] = None, b_opt: Optional[Optimizer] = None,
                 w_reg: Optional[Regularizer] = None, b_reg: Optional[Regularizer] = None):
        self.input_dim = int(input_dim)
        self.output_dim = int(output_dim)
        if w_init is None:
            w_init = HeNormal(gpu, self.input_dim)
        self.w = Parameter(gpu, shape=(self.output_dim, self.input_dim), initializer=w_init, opt=w_opt,
                           regularizer=w_reg)
        self.b = Parameter(gpu, shape=(self.output_dim,), initializer=b_init, opt=b_opt, regularizer=b_reg)

    def forward(self, x: Array) -> Array:
        return self.forward_act(x, _lib.ACT_NONE)

    def forward_act(self, x: Array, act: int) -> Array:
        """y = act(x W^T + b) in one kernel (the activation in the GEMM
        epilogue, same float32 ops as the separate ReLU / Sigmoid layer)."""
        y = Array(x._gpu, shape=(x.shape[0], self.output_dim))
        check(lib.vkc_dense_forward(x._h, _PREC[x._gpu.matmul_precision], x._dptr(), self.w.value._dptr(),
                                    self.b.value._dptr(), y._buf.ptr or 0, x.shape[0], x.shape[1],
                                    self.output_dim, act))
        y._written()
        return y

    def backward(self, dy: Array, need_dx: bool = True, accumulate: bool = True) -> Array:
        """Accumulate dW and db into the parameters' gradients (with
        ``accumulate`` False: overwrite them, as adding into zeroed gradients
        would) and return dx (not computed when ``need_dx`` is False, e.g. for
        the first layer)."""
        x = self._x
        dx = Array(dy._gpu, shape=(dy.shape[0], self.input_dim)) if need_dx else None
        wg = self.w.grad
        bg = self.b.grad
        check(lib.vkc_dense_backward_ex(
            dy._h, _PREC[dy._gpu.matmul_precision], x._dptr(), self.w.value._dptr(), dy._dptr(), None,
            _lib.ACT_NONE, None, dx._buf.ptr if dx is not None else None, wg._dptr() if wg is not None else None,
            bg._dptr() if bg is not None else None, dy.shape[0], self.input_dim, self.output_dim,
            1 if accumulate else 0))
        if wg is not None:
            wg._written()
        if bg is not None:
            bg._written()
        if dx is not None:
            dx._written()
        return dx

    def backward_act(self, dy_act: Array, act: int, y: Array, need_dx: bool = True,
                     accumulate: bool = True) -> Array:
        """The backward of the activation that follows this layer (output
        ``y``, gradient ``dy_act``) and then this layer's backward, with the
        activation derivative and the bias gradient in one kernel; the same
        float32 results as the two ``backward`` calls.  ``accumulate`` as for
        ``backward``."""
        x = self._x
        gpu = dy_act._gpu
        dy = Array(gpu, shape=(dy_act.shape[0], self.output_dim))
        dx = Array(gpu, shape=(dy_act.shape[0], self.input_dim)) if need_dx else None
        wg = self.w.grad
        bg = self.b.grad
        check(lib.vkc_dense_backward_ex(
            dy_act._h, _PREC[gpu.matmul_precision], x._dptr(), self.w.value._dptr(), dy_act._dptr(), y._dptr(),
            act, dy._buf.ptr or 0, dx._buf.ptr if dx is not None else None,
            wg._dptr() if wg is not None else None, bg._dptr() if bg is not None else None,
            dy_act.shape[0], self.input_dim, self.output_dim, 1 if accumulate else 0))
        dy._written()
        # held until the next call: a weight GEMM on a branch stream may still
        # read it after this returns (the caller may defer the join)
        self._act_dy = dy
        if wg is not None:
            wg._written()
        if bg is not None:
            bg._written()
        if dx is not None:
            dx._written()
        return dx

    def backward_chain(self, dy: Array, act: int, y: Array, accumulate: bool = True) -> Array:
        """This layer's backward followed by the backward of the activation
        below it (output ``y``): returns ``(dy W) * act'(y)``, the gradient
        the Dense layer under that activation receives, with the derivative
        applied inside the input-gradient GEMM; the same float32 results as
        ``backward`` then the activation's backward."""
        x = self._x
        gpu = dy._gpu
        dx = Array(gpu, shape=(dy.shape[0], self.input_dim))
        wg = self.w.grad
        bg = self.b.grad
        check(lib.vkc_dense_backward_chain(
            dy._h, _PREC[gpu.matmul_precision], x._dptr(), self.w.value._dptr(), dy._dptr(), y._dptr(), act,
            dx._buf.ptr or 0, wg._dptr() if wg is not None else None, bg._dptr() if bg is not None else None,
            dy.shape[0], self.input_dim, self.output_dim, 1 if accumulate else 0))
        if wg is not None:
            wg._written()
        if bg is not None:
            bg._written()
        dx._written()
        return dx

    def zero_grad(self):
        self.w.zero_grad()
        self.b.zero_grad()

    def update(self):
        self.w.update()
        self.b.update()


def _act_backward(act: int, y: Array, dy: Array) -> Array:
    dx = Array(dy._gpu, shape=dy.shape)
    check(lib.vkc_activation_backward(dy._h, act, y._dptr(), dy._dptr(), dx._buf.ptr or 0, dx._size))
    dx._written()
    return dx


class ReLU(Module):
    """max(x, 0); backward dy * max(sign(y), 0) (layers.py:158-210), one kernel."""

    act = _lib.ACT_RELU

    def forward(self, x: Array) -> Array:
        return x.max(0.0)

    def backward(self, dy: Array) -> Array:
        return _act_backward(_lib.ACT_RELU, self._y, dy)


class Sigmoid(Module):
    """1 / (1 + exp(0 - x)); backward dy * y * (1 - y) (layers.py:213-267)."""

    act = _lib.ACT_SIGMOID

    def forward(self, x: Array) -> Array:
        y = 0.0 - x
        y.exp(inplace=True)
        y += 1.0
        y = 1.0 / y
        return y

    def backward(self, dy: Array) -> Array:
        return _act_backward(_lib.ACT_SIGMOID, self._y, dy)


class Softmax(Module):
    """Softmax over axis 1; backward dy * y * (1 - y) (layers.py:270-323)."""

    def forward(self, x: Array) -> Array:
        if len(x.shape) == 2:
            y = Array(x._gpu, shape=x.shape)
            check(lib.vkc_softmax(x._h, x._dptr(), y._buf.ptr or 0, x.shape[0], x.shape[1]))
            y._written()
            return y
        X = x - x.maximum(axis=1, rebroadcast=True)
        X.exp(inplace=True)
        X /= X.sum(axis=1, rebroadcast=True)
        return X

    def backward(self, dy: Array) -> Array:
        # the reference's diagonal-only formula, same as Sigmoid's
        return _act_backward(_lib.ACT_SIGMOID, self._y, dy)
