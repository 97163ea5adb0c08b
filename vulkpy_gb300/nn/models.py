"""Sequential model (vulkpy/nn/models.py:15-105)."""
from __future__ import annotations

from typing import Iterable, Optional, Tuple, Union

import ctypes as C

from ..vkarray import Array
from ..graph import Graph
from .._lib import lib, check
from .. import _lib
from .core import Module, Loss
from .layers import Dense, ReLU, Sigmoid, Softmax, _PREC
from .optimizers import AdamState, SGDState

__all__ = ["Sequence", "CompiledStep"]


class Sequence:
    """Layers applied in order, trained against one loss.

    Execution differs from the reference only in how many kernels run, not
    in the float32 results: a Dense followed by ReLU or Sigmoid runs as one
    GEMM with the activation in its epilogue (the Dense pre-activation output
    is then not kept as ``dense._y``), backward the activation derivative
    and that Dense's bias gradient share one kernel, and the first layer's
    input gradient, which nothing consumes, is not computed.

    Like the reference, parameter regularizers are not applied by ``train``
    (vulkpy's Sequence never calls ``regular_grad``); pass
    ``apply_regularizers=True`` to add their gradients before the update."""

    def __init__(self, layers: Iterable[Module], loss: Loss, *, apply_regularizers: bool = False,
                 fuse: bool = True):
        self.L: Tuple[Module, ...] = tuple(layers)
        self.loss: Loss = loss
        self.apply_regularizers = apply_regularizers
        self.fuse = fuse

    def _stack_plan(self, x: Array):
        """The (Dense, activation or None) pairs when the whole model is a
        stack of Dense layers, each optionally followed by ReLU / Sigmoid, on
        the tensor-core path (run by one chained call), else None."""
        if not self.fuse or len(x.shape) != 2 or x._gpu.matmul_precision not in ("bf16", "bf16x3"):
            return None
        plan = []
        i, n = 0, len(self.L)
        while i < n:
            layer = self.L[i]
            if type(layer) is not Dense:
                return None
            nxt = self.L[i + 1] if i + 1 < n else None
            if type(nxt) in (ReLU, Sigmoid):
                plan.append((layer, nxt))
                i += 2
            else:
                plan.append((layer, None))
                i += 1
        return plan if len(plan) >= 2 else None

    def _forward_stack(self, x: Array, plan) -> Array:
        """The stack in one call (vkc_dense_stack_forward: each layer's
        split-K reduction also writes the next layer's operand pre-pass); the
        same float32 results and the same per-layer caches as the
        layer-by-layer path."""
        gpu = x._gpu
        dims = [x.shape[1]]
        for d, _ in plan:
            if d.input_dim != dims[-1]:
                raise ValueError(f"Dense input width {d.input_dim} does not match {dims[-1]}")
            dims.append(d.output_dim)
        ys = [Array(gpu, shape=(x.shape[0], d.output_dim)) for d, _ in plan]
        k = len(plan)
        ptrs = lambda v: (C.c_void_p * k)(*v)
        check(lib.vkc_dense_stack_forward(
            x._h, _PREC[gpu.matmul_precision], k, x._dptr(), x.shape[0], (C.c_int64 * (k + 1))(*dims),
            ptrs([d.w.value._dptr() for d, _ in plan]), ptrs([d.b.value._dptr() for d, _ in plan]),
            (C.c_int * k)(*[a.act if a is not None else _lib.ACT_NONE for _, a in plan]),
            ptrs([y._buf.ptr or 0 for y in ys])))
        inp = x
        for (d, a), y in zip(plan, ys):
            y._written()
            d._x = inp
            if a is None:
                d._y = y
            else:
                d._y = None
                a._x = None
                a._y = y
            inp = y
        return ys[-1]

    def _forward(self, x: Array) -> Array:
        plan = self._stack_plan(x)
        if plan is not None:
            return self._forward_stack(x, plan)
        i = 0
        n = len(self.L)
        while i < n:
            layer = self.L[i]
            nxt = self.L[i + 1] if i + 1 < n else None
            if (self.fuse and type(layer) is Dense and type(nxt) in (ReLU, Sigmoid) and len(x.shape) == 2):
                if len(x.shape) < 2:
                    raise ValueError("Input must have at least 2-dimensions.")
                layer._x = x
                layer._y = None
                y = layer.forward_act(x, nxt.act)
                nxt._x = None
                nxt._y = y
                x = y
                i += 2
                continue
            x = layer(x)
            i += 1
        return x

    def _backward(self, accumulate: bool = True, early_update: bool = False):
        """Backward through the layers; with ``accumulate`` False the Dense
        layers overwrite their gradients (each is written once per step)
        instead of adding to them.  ``early_update``: each Dense layer's
        optimizer step is issued on the side branch as soon as its gradients
        are (it waits there for them and for the layer's last use of its
        weights, the input-gradient GEMM), so only the first layer's step
        follows the backward on the main stream."""
        dx = self.loss.grad()
        # the Dense layers' weight GEMMs and bias sums stay on branch streams
        # until the whole backward is issued (joined back in the finally)
        # The gradients passed down are kept alive until then: a buffer freed
        # (stream-ordered, on the device's stream) while a branch still reads
        # it could be handed to the next allocation.
        h = dx._h
        keep = [dx]
        check(lib.vkc_side_defer(h, 1))
        try:
            self._backward_layers(dx, accumulate, keep, early_update)
        finally:
            check(lib.vkc_side_defer(h, 0))
            del keep

    def _update_early(self, dense: Dense):
        h = dense.w.value._h
        check(lib.vkc_side_begin(h))
        try:
            done = self._update_grouped([dense.w, dense.b])
        finally:
            check(lib.vkc_side_end(h))
        if not done:
            raise RuntimeError("early optimizer step without a shared Adam / SGD optimizer")

    def _backward_layers(self, dx, accumulate: bool, keep: list, early_update: bool = False):
        k = len(self.L) - 1
        while k >= 0:
            layer = self.L[k]
            prev = self.L[k - 1] if k >= 1 else None
            below = self.L[k - 2] if k >= 2 else None
            if (self.fuse and type(layer) is Dense and type(prev) in (ReLU, Sigmoid) and type(below) is Dense
                    and getattr(prev, "_y", None) is not None and len(dx.shape) == 2):
                # this layer's backward with the activation's below it in the
                # same GEMM: dx is already the lower Dense layer's dy
                dx = layer.backward_chain(dx, prev.act, prev._y, accumulate=accumulate)
                keep.append(dx)
                if early_update:
                    self._update_early(layer)
                k -= 2
                continue
            if (self.fuse and type(layer) in (ReLU, Sigmoid) and type(prev) is Dense
                    and getattr(layer, "_y", None) is not None
                    and len(dx.shape) == 2):
                # the activation's backward and the Dense bias sum in one kernel
                dx = prev.backward_act(dx, layer.act, layer._y, need_dx=k - 1 > 0, accumulate=accumulate)
                keep.append(dx)
                if early_update:
                    self._update_early(prev)
                k -= 2
                continue
            if type(layer) is Dense:
                dx = layer.backward(dx, need_dx=k > 0, accumulate=accumulate)
                if early_update:
                    self._update_early(layer)
            elif k == 0 and isinstance(layer, Dense):
                layer.backward(dx, need_dx=False)
            else:
                dx = layer.backward(dx)
            keep.append(dx)
            k -= 1

    def _overwrites_grads(self) -> bool:
        """True when one backward writes every gradient exactly once, so
        train() can overwrite gradients instead of zeroing then adding:
        only Dense / ReLU / Sigmoid / Softmax layers, no Dense twice."""
        dense = [L for L in self.L if type(L) is Dense]
        if len({id(L) for L in dense}) != len(dense):
            return False
        return all(type(L) in (Dense, ReLU, Sigmoid, Softmax) for L in self.L)

    def _params(self):
        """The trainable Parameters of the Dense layers, or None when another
        layer type (which may hold its own parameters) is present."""
        ps = []
        for _L in self.L:
            if type(_L) is Dense:
                ps.extend(p for p in (_L.w, _L.b) if p.grad is not None)
            elif not isinstance(_L, (ReLU, Sigmoid)) and (hasattr(_L, "w") or hasattr(_L, "b")):
                return None
        return ps

    def _zero_grad(self):
        # every gradient in one launch (the same zeros as Parameter.zero_grad)
        ps = self._params()
        if not ps:
            for _L in self.L:
                _L.zero_grad()
            return
        for _L in self.L:
            if type(_L) is not Dense:
                _L.zero_grad()
        gpu = ps[0].grad._gpu
        n = len(ps)
        check(lib.vkc_fill_f32_grouped(gpu._dev.h, (C.c_void_p * n)(*[p.grad._dptr() for p in ps]),
                                       (C.c_int64 * n)(*[p.grad._size for p in ps]), 0.0, n))
        for p in ps:
            p.grad._written()

    def _update(self):
        if self.apply_regularizers:
            for _L in self.L:
                for p in (getattr(_L, "w", None), getattr(_L, "b", None)):
                    if p is not None:
                        p.regular_grad()
        ps = self._params()
        if ps and self._update_grouped(ps):
            return
        for _L in self.L:
            _L.update()

    def _shares_one_optimizer(self) -> bool:
        """Every parameter under one Adam or one SGD optimizer (the grouped
        step's condition), on the device's own stream (branches need it)."""
        ps = self._params()
        if not ps:
            return False
        st = [p.opt_state for p in ps]
        if any(s.opt is not st[0].opt for s in st):
            return False
        if not (all(type(s) is AdamState for s in st) or all(type(s) is SGDState for s in st)):
            return False
        return ps[0].value._gpu._dev.own_stream()

    def _update_grouped(self, ps) -> bool:
        """One launch for every parameter when they share one Adam or one SGD
        optimizer (per tensor the same arithmetic as Parameter.update)."""
        st = [p.opt_state for p in ps]
        opt = st[0].opt
        if any(s.opt is not opt for s in st):
            return False
        gpu = ps[0].value._gpu
        n = len(ps)
        vals = (C.c_void_p * n)(*[p.value._dptr() for p in ps])
        grads = (C.c_void_p * n)(*[p.grad._dptr() for p in ps])
        sizes = (C.c_int64 * n)(*[p.value._size for p in ps])
        if all(type(s) is AdamState for s in st):
            check(lib.vkc_adam_update_grouped(
                gpu._dev.h, vals, grads, (C.c_void_p * n)(*[s.m._dptr() for s in st]),
                (C.c_void_p * n)(*[s.v._dptr() for s in st]), (C.c_void_p * n)(*[s._powers._dptr() for s in st]),
                sizes, n, float(opt.lr), float(opt.beta1), float(opt.beta2), float(opt.eps)))
            for s in st:
                s.beta1t *= opt.beta1
                s.beta2t *= opt.beta2
                s._powers._written()
                s.m._written()
                s.v._written()
        elif all(type(s) is SGDState for s in st):
            check(lib.vkc_sgd_update_grouped(gpu._dev.h, vals, grads, sizes, float(opt.lr), n))
        else:
            return False
        for p in ps:
            p.value._written()
        return True

    def train(self, x: Array, y: Array) -> Tuple[Array, Array]:
        """One step: forward, loss, zero_grad, backward, update (models.py:55-78).
        When every gradient is written exactly once by the backward, the
        zeroing is folded into it (gradients overwritten, the same values)."""
        _y = self._forward(x)
        _loss = self.loss(_y, y)
        if self.fuse and self._overwrites_grads():
            early = not self.apply_regularizers and self._shares_one_optimizer()
            self._backward(accumulate=False, early_update=early)
            if not early:
                self._update()
        else:
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

    def compile(self, x: Array, y: Array) -> "CompiledStep":
        """Capture one ``train(x, y)`` step as a CUDA graph.

        Returns a callable that replays the step on the device with one
        launch; ``x`` and ``y`` are the step's input buffers (write the next
        batch into them in place, e.g. ``x[:] = batch``).  The first call of
        ``train`` must already have run (kernel set-up is not captured).
        Optimizer states keep their running powers on the device, so replays
        match eager steps exactly; host-side mirrors of those counters (e.g.
        ``AdamState.beta1t``) are not advanced by replays."""
        g = Graph(x._gpu)
        with g:
            _y, _loss = self.train(x, y)
        return CompiledStep(g, _y, _loss, (x, y))


class CompiledStep:
    """A captured training step: ``step()`` -> (prediction, loss) arrays,
    rewritten in place by every call."""

    def __init__(self, graph: Graph, pred: Array, loss: Array, inputs):
        self.graph = graph
        self.pred = pred
        self.loss = loss
        self.inputs = inputs

    def __call__(self) -> Tuple[Array, Array]:
        self.graph.launch(flush=self.inputs)
        return self.pred, self.loss
