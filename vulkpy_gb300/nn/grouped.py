"""
Many independent models trained with grouped launches.

The reference trains each model on its own (every Dense layer of every model
is a separate job, nn/layers.py:94-141).  ``GroupedSequence`` runs one
training step of a list of ``Sequence`` models -- each with its own layer
widths and batch size -- as a handful of launches for all of them: one
grouped GEMM per layer and direction (bias and ReLU fused into the forward
epilogue, the ReLU derivative fused into the backward one), one grouped loss
kernel and one grouped bias-gradient kernel per layer.  The SGD step is
fused: each weight moves in the epilogue of the GEMM that computes its
gradient and each bias in its gradient's column-sum kernel, after the
gradient is stored and in the arithmetic of the separate SGD kernel.
The step is graph-capturable (``Sequence.compile``-style: capture
``train(xs, ys)`` once and replay).

Supported models: ``Sequence([Dense, (ReLU,) Dense, (ReLU,) ..., Dense],
MSELoss())`` with SGD optimizers -- the batched workload of 64 uneven
2-layer MLPs.  Parameters after a step equal those of calling each model's
own ``train`` (fp32 and split-bf16x3 when those calls do not split K); the
loss values agree to float32 rounding (different summation order).  The
models' per-layer caches (``_x``/``_y``) are not updated.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence as Seq, Tuple

import numpy as np

from ..vkarray import Array
from .._lib import lib, check, GemmProblem, GemmUpdate
from .. import _lib
from .layers import Dense, ReLU
from .losses import MSELoss
from .models import Sequence
from .optimizers import SGDState

__all__ = ["GroupedSequence"]

_PREC = {"fp32": _lib.MM_FP32, "bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}


def _ptrs(arrs) -> "C.Array":
    return (C.c_void_p * len(arrs))(*[a for a in arrs])


class GroupedSequence:
    """Train several ``Sequence`` models of different sizes together."""

    def __init__(self, models: Seq[Sequence]):
        self.models: List[Sequence] = list(models)
        if not self.models:
            raise ValueError("no models")
        self._plan = [self._layers(m) for m in self.models]
        pattern = [tuple(relu for _, relu in p) for p in self._plan]
        if any(p != pattern[0] for p in pattern):
            raise ValueError("grouped models must have the same layer pattern")
        self.gpu = self.models[0].L[0].w.value._gpu

    @staticmethod
    def _layers(model: Sequence):
        if not isinstance(model.loss, MSELoss):
            raise NotImplementedError("GroupedSequence supports MSELoss")
        if model.loss.scale_backward is None:
            raise NotImplementedError("GroupedSequence supports MSELoss(reduce='mean')")
        if model.apply_regularizers:
            raise NotImplementedError("GroupedSequence does not apply regularizers")
        out: List[Tuple[Dense, bool]] = []
        L = list(model.L)
        i = 0
        while i < len(L):
            if type(L[i]) is not Dense:
                raise NotImplementedError(f"GroupedSequence supports Dense and ReLU layers, got {type(L[i]).__name__}")
            relu = i + 1 < len(L) and type(L[i + 1]) is ReLU
            for p in (L[i].w, L[i].b):
                if not isinstance(p.opt_state, SGDState):
                    raise NotImplementedError("GroupedSequence supports SGD")
            out.append((L[i], relu))
            i += 2 if relu else 1
        if out[-1][1]:
            raise NotImplementedError("the last layer must be a Dense without activation")
        return out

    def _gemm(self, problems: List[GemmProblem], updates: List[GemmUpdate] = None):
        arr = (GemmProblem * len(problems))(*problems)
        if updates is None:
            check(lib.vkc_gemm_grouped(self.gpu._dev.h, _PREC[self.gpu.matmul_precision], arr, len(problems)))
        else:
            upd = (GemmUpdate * len(updates))(*updates)
            check(lib.vkc_gemm_grouped_update(self.gpu._dev.h, _PREC[self.gpu.matmul_precision], arr, upd,
                                              len(problems)))

    def train(self, xs: Seq[Array], ys: Seq[Array]) -> Tuple[List[Array], Array]:
        """One step for every model: forward, MSE loss, backward, SGD.
        Returns the predictions and the losses (an Array of shape (models,))."""
        if len(xs) != len(self.models) or len(ys) != len(self.models):
            raise ValueError("one input and one target per model")
        gpu = self.gpu
        n = len(self.models)
        nl = len(self._plan[0])
        acts = [[x] for x in xs]        # acts[m][l]: input of layer l (post-activation)
        # ---- forward: one grouped GEMM per layer
        for l in range(nl):
            probs = []
            outs = []
            for m in range(n):
                d, relu = self._plan[m][l]
                x = acts[m][l]
                if len(x.shape) != 2 or x.shape[1] != d.input_dim:
                    raise ValueError(f"model {m} layer {l}: input shape {x.shape} does not match {d.input_dim}")
                y = Array(gpu, shape=(x.shape[0], d.output_dim))
                outs.append(y)
                probs.append(GemmProblem(
                    ta=0, tb=1, m=x.shape[0], n=d.output_dim, k=d.input_dim, alpha=1.0, beta=0.0,
                    a=x._dptr(), lda=d.input_dim, b=d.w.value._dptr(), ldb=d.input_dim, c=y._buf.ptr or 0,
                    ldc=d.output_dim, bias=d.b.value._dptr(), act=_lib.ACT_RELU if relu else _lib.ACT_NONE,
                    relu_mask=None))
            self._gemm(probs)
            for m, y in enumerate(outs):
                y._written()
                acts[m].append(y)
        preds = [a[-1] for a in acts]
        # ---- loss and its gradient
        losses = Array(gpu, shape=(n,))
        dys = [Array(gpu, shape=p.shape) for p in preds]
        for y in ys:
            y._dptr()
        check(lib.vkc_mse_grouped(gpu._dev.h, _ptrs([p._dptr() for p in preds]), _ptrs([y._dptr() for y in ys]),
                                  _ptrs([d._buf.ptr or 0 for d in dys]),
                                  (C.c_int64 * n)(*[p.shape[0] for p in preds]),
                                  (C.c_int64 * n)(*[p.shape[1] for p in preds]), losses._buf.ptr or 0, n))
        losses._written()
        for d in dys:
            d._written()
        # ---- backward
        for l in range(nl - 1, -1, -1):
            dense = [self._plan[m][l][0] for m in range(n)]
            # bias gradients (overwrite: db = 0 + sum_b dy), then b += (-lr) db
            check(lib.vkc_colsum_update_grouped(gpu._dev.h, _ptrs([dy._dptr() for dy in dys]),
                                                _ptrs([d.b.grad._dptr() for d in dense]),
                                                (C.c_int64 * n)(*[dy.shape[0] for dy in dys]),
                                                (C.c_int64 * n)(*[d.output_dim for d in dense]), n, 1,
                                                _ptrs([d.b.value._dptr() for d in dense]),
                                                (C.c_float * n)(*[-d.b.opt_state.opt.lr for d in dense])))
            probs = []
            upds = []
            nxt = []
            for m in range(n):
                d = dense[m]
                dy, x = dys[m], acts[m][l]
                # dW = dy^T x (the gradient is overwritten, as zero_grad + accumulate would give)
                probs.append(GemmProblem(
                    ta=1, tb=0, m=d.output_dim, n=d.input_dim, k=dy.shape[0], alpha=1.0, beta=0.0,
                    a=dy._dptr(), lda=d.output_dim, b=x._dptr(), ldb=d.input_dim, c=d.w.grad._dptr(),
                    ldc=d.input_dim, bias=None, act=_lib.ACT_NONE, relu_mask=None))
                # then W += (-lr) dW in the same GEMM (its dx problem below reads W before the step)
                upds.append(GemmUpdate(value=d.w.value._dptr(), scale=-d.w.opt_state.opt.lr))
                if l > 0:
                    # dx = (dy W) * relu'(x): x is the previous layer's ReLU output
                    relu_prev = self._plan[m][l - 1][1]
                    dx = Array(gpu, shape=(dy.shape[0], d.input_dim))
                    nxt.append(dx)
                    probs.append(GemmProblem(
                        ta=0, tb=0, m=dy.shape[0], n=d.input_dim, k=d.output_dim, alpha=1.0, beta=0.0,
                        a=dy._dptr(), lda=d.output_dim, b=d.w.value._dptr(), ldb=d.input_dim, c=dx._buf.ptr or 0,
                        ldc=d.input_dim, bias=None, act=_lib.ACT_NONE,
                        relu_mask=x._dptr() if relu_prev else None))
                    upds.append(GemmUpdate(value=None, scale=0.0))
            self._gemm(probs, upds)
            for d in dense:
                d.w.grad._written()
                d.b.grad._written()
                d.w.value._written()
                d.b.value._written()
            if l > 0:
                for dx in nxt:
                    dx._written()
                dys = nxt
        return preds, losses
