"""
torch.autograd.Function wrappers over the library's hand-written kernels.

Forward and backward of Dense (with its activation fused into the GEMM
epilogue), the standalone ReLU / Sigmoid / Softmax layers and every loss
(cross entropy, softmax cross entropy, MSE, Huber and weighted mixes of
them) run as this library's CUDA kernels on torch tensors, on torch's
current stream; torch only provides memory, streams and the autograd tape.
The math is vulkpy's (vulkpy/nn/layers.py:71-323, vulkpy/nn/losses.py:40-458).
float64 tensors run the same kernels instantiated in double, so gradients
can be checked against float64 finite differences.

Where vulkpy's backward is not the derivative of its forward, the default
here is the exact gradient and ``grad="vulkpy"`` reproduces the reference:
  * Softmax: vulkpy keeps only the Jacobian's diagonal, dy y (1 - y)
    (layers.py:302-323); exact: y (dy - sum(dy y)).
  * Huber: vulkpy returns clamp(x - y, -1, 1) (losses.py:376-393) for the
    forward 0.5 min(|d|, d^2), whose derivative is 0.5 sign(d) for |d| > 1.

>>> import torch, vulkpy_gb300.autograd as A
>>> y = A.dense(x, W, b, act="relu")           # x (B, in), W (out, in), b (out,)
>>> loss = A.softmax_cross_entropy(logits, onehot)
>>> loss = A.mix([(0.3, "mse"), (0.7, "huber")], pred, target)
>>> loss.backward()
"""
from __future__ import annotations

import contextlib
import ctypes as C

import torch

from . import _lib
from ._lib import lib, check
from .vkarray import _Device

__all__ = ["dense", "relu", "sigmoid", "softmax", "cross_entropy", "softmax_cross_entropy", "mse", "huber", "mix",
           "DenseFunction", "ActivationFunction", "SoftmaxFunction", "LossFunction"]

_ACTS = {None: _lib.ACT_NONE, "none": _lib.ACT_NONE, "relu": _lib.ACT_RELU, "sigmoid": _lib.ACT_SIGMOID}
_PREC = {"fp32": _lib.MM_FP32, "bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}
_LOSSES = {"ce": _lib.LOSS_CE, "cross_entropy": _lib.LOSS_CE, "sce": _lib.LOSS_SCE,
           "softmax_cross_entropy": _lib.LOSS_SCE, "mse": _lib.LOSS_MSE, "huber": _lib.LOSS_HUBER}


# cudaStreamLegacy: the legacy default stream by an explicit handle.  torch's
# default stream has handle 0, which vkc_device_set_stream would read as
# "back to the device's own stream" -- a non-blocking stream that does not
# wait for torch's work.
_CUDA_STREAM_LEGACY = 1


@contextlib.contextmanager
def _on_torch_stream(t: torch.Tensor):
    """The device handle for t's GPU, with work routed to torch's current
    stream (so it is ordered with torch's own kernels on the tensors)."""
    if not t.is_cuda or t.dtype not in (torch.float32, torch.float64):
        raise TypeError("vulkpy_gb300.autograd needs float32 (or float64, for checking) CUDA tensors")
    dev = _Device.get(t.device.index or 0, 0.0)
    stream = torch.cuda.current_stream(t.device).cuda_stream or _CUDA_STREAM_LEGACY
    check(lib.vkc_device_set_stream(dev.h, stream))
    try:
        yield dev.h
    finally:
        check(lib.vkc_device_set_stream(dev.h, None))


def _p(t: torch.Tensor) -> int:
    return t.data_ptr()


class DenseFunction(torch.autograd.Function):
    """y = act(x W^T + b).  float64 tensors run the float64 kernels."""

    @staticmethod
    def forward(ctx, x, W, b, act: int, precision: int):
        x, W, b = x.contiguous(), W.contiguous(), b.contiguous()
        B, I = x.shape
        O = W.shape[0]
        y = torch.empty((B, O), device=x.device, dtype=x.dtype)
        with _on_torch_stream(x) as h:
            if x.dtype == torch.float64:
                check(lib.vkc_dense_forward_f64(h, _p(x), _p(W), _p(b), _p(y), B, I, O, act))
            else:
                check(lib.vkc_dense_forward(h, precision, _p(x), _p(W), _p(b), _p(y), B, I, O, act))
        ctx.save_for_backward(x, W, y)
        ctx.act, ctx.precision = act, precision
        return y

    @staticmethod
    def backward(ctx, dy):
        x, W, y = ctx.saved_tensors
        dy = dy.contiguous()
        B, I = x.shape
        O = W.shape[0]
        f64 = x.dtype == torch.float64
        dW = torch.zeros_like(W)
        db = torch.zeros((O,), device=x.device, dtype=x.dtype)
        dx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        with _on_torch_stream(x) as h:
            g = dy
            if ctx.act != _lib.ACT_NONE:
                g = torch.empty_like(dy)
                fn = lib.vkc_activation_backward_f64 if f64 else lib.vkc_activation_backward
                check(fn(h, ctx.act, _p(y), _p(dy), _p(g), g.numel()))
            pdx = _p(dx) if dx is not None else None
            if f64:
                check(lib.vkc_dense_backward_f64(h, _p(x), _p(W), _p(g), pdx, _p(dW), _p(db), B, I, O))
            else:
                check(lib.vkc_dense_backward(h, ctx.precision, _p(x), _p(W), _p(g), pdx, _p(dW), _p(db), B, I, O))
        return dx, dW, db, None, None


class ActivationFunction(torch.autograd.Function):
    """Standalone ReLU / Sigmoid (layers.py:158-267): forward and backward
    kernels, the backward from the saved output."""

    @staticmethod
    def forward(ctx, x, act: int):
        x = x.contiguous()
        y = torch.empty_like(x)
        with _on_torch_stream(x) as h:
            fn = lib.vkc_activation_forward_f64 if x.dtype == torch.float64 else lib.vkc_activation_forward
            check(fn(h, act, _p(x), _p(y), x.numel()))
        ctx.save_for_backward(y)
        ctx.act = act
        return y

    @staticmethod
    def backward(ctx, dy):
        (y,) = ctx.saved_tensors
        dy = dy.contiguous()
        dx = torch.empty_like(y)
        with _on_torch_stream(y) as h:
            fn = lib.vkc_activation_backward_f64 if y.dtype == torch.float64 else lib.vkc_activation_backward
            check(fn(h, ctx.act, _p(y), _p(dy), _p(dx), dx.numel()))
        return dx, None


class SoftmaxFunction(torch.autograd.Function):
    """Softmax over the last axis of a 2-D tensor (layers.py:270-323).
    Backward: the full Jacobian-vector product, or with ``exact=False``
    the reference's diagonal-only dy y (1 - y)."""

    @staticmethod
    def forward(ctx, x, exact: bool):
        x = x.contiguous()
        y = torch.empty_like(x)
        R, Cn = x.shape
        with _on_torch_stream(x) as h:
            fn = lib.vkc_softmax_f64 if x.dtype == torch.float64 else lib.vkc_softmax
            check(fn(h, _p(x), _p(y), R, Cn))
        ctx.save_for_backward(y)
        ctx.exact = exact
        return y

    @staticmethod
    def backward(ctx, dy):
        (y,) = ctx.saved_tensors
        dy = dy.contiguous()
        dx = torch.empty_like(y)
        f64 = y.dtype == torch.float64
        with _on_torch_stream(y) as h:
            if ctx.exact:
                fn = lib.vkc_softmax_backward_f64 if f64 else lib.vkc_softmax_backward
                check(fn(h, _p(y), _p(dy), _p(dx), y.shape[0], y.shape[1]))
            else:
                fn = lib.vkc_activation_backward_f64 if f64 else lib.vkc_activation_backward
                check(fn(h, _lib.ACT_SIGMOID, _p(y), _p(dy), _p(dx), dx.numel()))
        return dx, None


class LossFunction(torch.autograd.Function):
    """sum_j coeff_j * reduce_j(loss_j(x, y)) over 2-D (batch, features)
    tensors, reduce = mean or sum over the batch (ReduceLoss,
    losses.py:40-92; MixLoss, losses.py:396-458).  One kernel per term
    forward (the per-row losses) and one fused kernel for the whole
    backward.  ``terms`` is a tuple of (coeff, kind, reduce)."""

    @staticmethod
    def forward(ctx, x, y, terms, huber_exact: bool):
        x, y = x.contiguous(), y.contiguous()
        if x.dim() != 2 or x.shape != y.shape:
            raise ValueError("losses take 2-D x and y of the same shape")
        R, Cn = x.shape
        f64 = x.dtype == torch.float64
        rows_fn = lib.vkc_loss_rows_f64 if f64 else lib.vkc_loss_rows
        total = None
        p = None
        with _on_torch_stream(x) as h:
            for coeff, kind, reduce in terms:
                rows = torch.empty((R,), device=x.device, dtype=x.dtype)
                p_out = None
                if kind == _lib.LOSS_SCE:
                    if p is None:
                        p = torch.empty_like(x)
                    p_out = _p(p)
                check(rows_fn(h, kind, _p(x), _p(y), _p(rows), p_out, R, Cn))
                val = rows.mean() if reduce == "mean" else rows.sum()
                val = val * coeff if len(terms) > 1 else val
                total = val if total is None else total + val
        ctx.save_for_backward(x, y, p if p is not None else x)
        ctx.terms, ctx.huber_exact, ctx.has_p = terms, huber_exact, p is not None
        return total

    @staticmethod
    def backward(ctx, dloss):
        x, y, p = ctx.saved_tensors
        n = len(ctx.terms)
        kinds = (C.c_int * n)(*[k for _, k, _ in ctx.terms])
        coeffs = (C.c_double * n)(*[float(c) for c, _, _ in ctx.terms])
        scales = (C.c_double * n)(*[1.0 / x.shape[0] if r == "mean" else 1.0 for _, _, r in ctx.terms])
        dx = torch.empty_like(x)
        f64 = x.dtype == torch.float64
        with _on_torch_stream(x) as h:
            fn = lib.vkc_loss_backward_f64 if f64 else lib.vkc_loss_backward
            check(fn(h, n, kinds, coeffs, scales, 1 if ctx.huber_exact else 0, _p(x), _p(y),
                     _p(p) if ctx.has_p else None, _p(dx), dx.numel()))
        return dx * dloss, None, None, None


def _loss_terms(spec, reduce):
    terms = []
    for coeff, kind in spec:
        k = _LOSSES[kind] if isinstance(kind, str) else int(kind)
        terms.append((float(coeff), k, reduce))
    return tuple(terms)


def dense(x, W, b, act=None, precision: str = "fp32"):
    return DenseFunction.apply(x, W, b, _ACTS[act], _PREC[precision])


def relu(x):
    return ActivationFunction.apply(x, _lib.ACT_RELU)


def sigmoid(x):
    return ActivationFunction.apply(x, _lib.ACT_SIGMOID)


def softmax(x, grad: str = "exact"):
    """Row softmax; ``grad="vulkpy"`` uses the reference's diagonal backward."""
    return SoftmaxFunction.apply(x, grad != "vulkpy")


def cross_entropy(x, y, reduce: str = "mean"):
    """-y log(x + 1e-8) summed per row, reduced over the batch (x: probabilities)."""
    return LossFunction.apply(x, y, _loss_terms([(1.0, "ce")], reduce), True)


def softmax_cross_entropy(x, y, reduce: str = "mean"):
    return LossFunction.apply(x, y, _loss_terms([(1.0, "sce")], reduce), True)


def mse(x, y, reduce: str = "mean"):
    return LossFunction.apply(x, y, _loss_terms([(1.0, "mse")], reduce), True)


def huber(x, y, reduce: str = "mean", grad: str = "exact"):
    """0.5 min(|y - x|, (y - x)^2); ``grad="vulkpy"`` gives the reference's
    clamp(x - y, -1, 1) backward."""
    return LossFunction.apply(x, y, _loss_terms([(1.0, "huber")], reduce), grad != "vulkpy")


def mix(spec, x, y, reduce: str = "mean", huber_grad: str = "exact"):
    """Weighted sum of losses, ``spec`` = [(coeff, kind), ...] with kind one
    of "ce", "sce", "mse", "huber" (MixLoss, losses.py:396-458); the
    backward is one fused kernel."""
    if not spec:
        raise ValueError("losses should not empty")
    return LossFunction.apply(x, y, _loss_terms(spec, reduce), huber_grad != "vulkpy")
