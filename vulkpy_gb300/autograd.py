"""
torch.autograd.Function wrappers over the library's hand-written kernels.

Forward and backward of Dense (with its activation fused into the GEMM
epilogue), the activations' backward and the softmax-cross-entropy / MSE
losses run as this library's CUDA kernels on torch tensors, on torch's
current stream; torch only provides memory, streams and the autograd tape.
The math is vulkpy's (vulkpy/nn/layers.py:71-141, 158-267,
vulkpy/nn/losses.py:179-320), with the true softmax Jacobian handled by the
fused softmax-cross-entropy loss.

>>> import torch, vulkpy_gb300.autograd as A
>>> y = A.dense(x, W, b, act="relu")           # x (B, in), W (out, in), b (out,)
>>> loss = A.softmax_cross_entropy(logits, onehot)
>>> loss.backward()
"""
from __future__ import annotations

import contextlib

import torch

from . import _lib
from ._lib import lib, check
from .vkarray import _Device

__all__ = ["dense", "softmax_cross_entropy", "mse", "DenseFunction", "SoftmaxCrossEntropyFunction",
           "MSEFunction"]

_ACTS = {None: _lib.ACT_NONE, "none": _lib.ACT_NONE, "relu": _lib.ACT_RELU, "sigmoid": _lib.ACT_SIGMOID}
_PREC = {"fp32": _lib.MM_FP32, "bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}


@contextlib.contextmanager
def _on_torch_stream(t: torch.Tensor):
    """The device handle for t's GPU, with work routed to torch's stream."""
    if not t.is_cuda or t.dtype not in (torch.float32, torch.float64):
        raise TypeError("vulkpy_gb300.autograd needs float32 (or float64, for checking) CUDA tensors")
    dev = _Device.get(t.device.index or 0, 0.0)
    check(lib.vkc_device_set_stream(dev.h, torch.cuda.current_stream(t.device).cuda_stream))
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


class SoftmaxCrossEntropyFunction(torch.autograd.Function):
    """mean over rows of sum_c -y log(softmax(x) + 1e-8)."""

    @staticmethod
    def forward(ctx, x, y):
        x, y = x.contiguous(), y.contiguous()
        R, Cn = x.shape
        rows = torch.empty((R,), device=x.device, dtype=x.dtype)
        p = torch.empty_like(x)
        with _on_torch_stream(x) as h:
            fn = lib.vkc_cross_entropy_f64 if x.dtype == torch.float64 else lib.vkc_cross_entropy
            check(fn(h, _p(x), _p(y), _p(rows), _p(p), R, Cn, 1))
        ctx.save_for_backward(p, y)
        return rows.mean()

    @staticmethod
    def backward(ctx, dloss):
        p, y = ctx.saved_tensors
        dx = torch.empty_like(p)
        with _on_torch_stream(p) as h:
            fn = lib.vkc_softmax_ce_backward_f64 if p.dtype == torch.float64 else lib.vkc_softmax_ce_backward
            check(fn(h, _p(p), _p(y), _p(dx), dx.numel(), 1.0 / p.shape[0]))
        return dx * dloss, None


class MSEFunction(torch.autograd.Function):
    """mean over rows of sum_c (y - x)^2 (losses.py:252-320)."""

    @staticmethod
    def forward(ctx, x, y):
        ctx.save_for_backward(x, y)
        d = torch.empty_like(x)
        with _on_torch_stream(x) as h:
            check(lib.vkc_binary(h, _lib.SUB, _p(y.contiguous()), _p(x.contiguous()), _p(d), d.numel()))
            check(lib.vkc_binary(h, _lib.MUL, _p(d), _p(d), _p(d), d.numel()))
        return d.sum(dim=1).mean()

    @staticmethod
    def backward(ctx, dloss):
        x, y = ctx.saved_tensors
        dx = torch.empty_like(x)
        with _on_torch_stream(x) as h:
            check(lib.vkc_binary(h, _lib.SUB, _p(x.contiguous()), _p(y.contiguous()), _p(dx), dx.numel()))
            check(lib.vkc_binary_scalar(h, _lib.MUL, _p(dx), 2.0 / x.shape[0], _p(dx), dx.numel()))
        return dx * dloss, None


def dense(x, W, b, act=None, precision: str = "fp32"):
    return DenseFunction.apply(x, W, b, _ACTS[act], _PREC[precision])


def softmax_cross_entropy(x, y):
    return SoftmaxCrossEntropyFunction.apply(x, y)


def mse(x, y):
    return MSEFunction.apply(x, y)
