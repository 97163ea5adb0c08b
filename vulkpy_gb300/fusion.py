"""
Fusion of elementwise op chains into one kernel (no counterpart in vulkpy,
which runs one shader per op and writes every intermediate to memory).

>>> @vk.fusion.fuse
... def f(x, y):
...     t = x * 1.5 + y
...     return t.tanh().exp() - y
>>> z = f(a, b)            # one kernel: reads a, b once, writes z once

The function is traced once per input shape with symbolic arrays that
support the same-shape elementwise subset of the Array API (+ - * / **,
max/min, the 20 math functions, clamp, scalar operands on either side,
in-place forms).  The trace becomes straight-line CUDA C, compiled at run
time for this GPU with FMA contraction off, so every op rounds exactly as
the one-op kernels do and the fused result is bit-identical to running the
ops one by one.  Python scalars in the function are compile-time constants.
"""
from __future__ import annotations

import ctypes as C
import functools
import hashlib
import math
import struct
from typing import Callable, Dict, List, Tuple

import numpy as np

from ._lib import lib, check
from .vkarray import Array

__all__ = ["fuse", "FusedFunction"]

_MAX_IN, _MAX_OUT = 8, 4

_UNARY = {
    "abs": "fabsf({})", "sign": "vkc_sign({})", "sin": "sinf({})", "cos": "cosf({})", "tan": "tanf({})",
    "asin": "asinf({})", "acos": "acosf({})", "atan": "atanf({})", "sinh": "sinhf({})", "cosh": "coshf({})",
    "tanh": "tanhf({})", "asinh": "asinhf({})", "acosh": "acoshf({})", "atanh": "atanhf({})",
    "exp": "expf({})", "log": "logf({})", "exp2": "exp2f({})", "log2": "log2f({})", "sqrt": "sqrtf({})",
    "invsqrt": "(1.0f / sqrtf({}))",
}


def _lit(s) -> str:
    """Exact float32 literal."""
    f = float(np.float32(s))
    if math.isfinite(f):
        return float.hex(f) + "f"
    bits = struct.unpack("<I", struct.pack("<f", f))[0]
    return f"__int_as_float(0x{bits:08x})"


class _Trace:
    def __init__(self, shape):
        self.shape = tuple(shape)
        self.lines: List[str] = []
        self.inputs: List[Array] = []
        self.n = 0

    def temp(self, expr: str) -> "_Sym":
        name = f"t{self.n}"
        self.n += 1
        self.lines.append(f"  const float {name} = {expr};")
        return _Sym(self, name)

    def input(self, arr: Array) -> "_Sym":
        for k, a in enumerate(self.inputs):
            if a is arr:
                return _Sym(self, f"x[{k}]")
        if len(self.inputs) >= _MAX_IN:
            raise ValueError(f"a fused function can read at most {_MAX_IN} arrays")
        if tuple(arr.shape) != self.shape:
            raise ValueError(f"fused operands must share one shape: {arr.shape} vs {self.shape}")
        self.inputs.append(arr)
        return _Sym(self, f"x[{len(self.inputs) - 1}]")


class _Sym:
    """Symbolic array inside a trace."""

    def __init__(self, tr: _Trace, ref: str):
        self._tr = tr
        self._ref = ref

    @property
    def shape(self):
        return self._tr.shape

    def _arg(self, o) -> str:
        if isinstance(o, _Sym):
            if o._tr is not self._tr:
                raise ValueError("operands from different traces")
            return o._ref
        if isinstance(o, Array):
            return self._tr.input(o)._ref
        return _lit(o)

    def _bin(self, o, fmt: str) -> "_Sym":
        return self._tr.temp(fmt.format(a=self._ref, b=self._arg(o)))

    def __add__(self, o): return self._bin(o, "{a} + {b}")
    def __sub__(self, o): return self._bin(o, "{a} - {b}")
    def __mul__(self, o): return self._bin(o, "{a} * {b}")
    def __truediv__(self, o): return self._bin(o, "{a} / {b}")
    def __radd__(self, o): return self._bin(o, "{a} + {b}")
    def __rmul__(self, o): return self._bin(o, "{a} * {b}")
    def __rsub__(self, o): return self._bin(o, "{b} - {a}")
    def __rtruediv__(self, o): return self._bin(o, "{b} / {a}")
    __iadd__, __isub__, __imul__, __itruediv__ = __add__, __sub__, __mul__, __truediv__

    def __pow__(self, o):
        if not isinstance(o, (_Sym, Array)) and float(np.float32(o)) == 2.0:
            return self._bin(o, "{a} * {a}")        # exact square, as the one-op kernel
        return self._bin(o, "powf({a}, {b})")

    __ipow__ = __pow__

    def __rpow__(self, o):
        return self._bin(o, "powf({b}, {a})")

    def max(self, o, inplace=False): return self._bin(o, "fmaxf({a}, {b})")
    def min(self, o, inplace=False): return self._bin(o, "fminf({a}, {b})")

    def clamp(self, lo, hi, inplace=False):
        return self._tr.temp(f"fminf(fmaxf({self._ref}, {self._arg(lo)}), {self._arg(hi)})")

    def __getattr__(self, name):
        if name in _UNARY:
            fmt = _UNARY[name]
            return lambda inplace=False: self._tr.temp(fmt.format(self._ref))
        raise AttributeError(name)


_PRELUDE = r"""
struct P { const float* in[8]; float* out[4]; unsigned long long n; };
__device__ __forceinline__ float vkc_sign(float v) { return v > 0.f ? 1.f : (v < 0.f ? -1.f : v); }
"""


def _source(name: str, tr: _Trace, outs: List[str], n_in: int) -> str:
    body = "\n".join(tr.lines)
    ret = "\n".join(f"  y[{j}] = {r};" for j, r in enumerate(outs))
    lanes = []
    for lane in "xyzw":
        lanes.append(
            "    {\n      float x[%d], y[%d];\n%s\n      body(x, y);\n%s\n    }" % (
                max(1, n_in), len(outs),
                "\n".join(f"      x[{k}] = v{k}.{lane};" for k in range(n_in)),
                "\n".join(f"      r{j}.{lane} = y[{j}];" for j in range(len(outs)))))
    return _PRELUDE + f"""
__device__ __forceinline__ void body(const float* x, float* y) {{
{body}
{ret}
}}
extern "C" __global__ void __launch_bounds__(256) {name}(P p) {{
  const unsigned long long n4 = p.n >> 2;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (unsigned long long i = tid; i < n4; i += stride) {{
{chr(10).join(f"    const float4 v{k} = reinterpret_cast<const float4*>(p.in[{k}])[i];" for k in range(n_in))}
{chr(10).join(f"    float4 r{j};" for j in range(len(outs)))}
{chr(10).join(lanes)}
{chr(10).join(f"    reinterpret_cast<float4*>(p.out[{j}])[i] = r{j};" for j in range(len(outs)))}
  }}
  const unsigned long long t = (n4 << 2) + tid;
  if (t < p.n) {{
    float x[{max(1, n_in)}], y[{len(outs)}];
{chr(10).join(f"    x[{k}] = p.in[{k}][t];" for k in range(n_in))}
    body(x, y);
{chr(10).join(f"    p.out[{j}][t] = y[{j}];" for j in range(len(outs)))}
  }}
}}
"""


class FusedFunction:
    """A traced, compiled elementwise function; see :func:`fuse`."""

    def __init__(self, fn: Callable):
        self.fn = fn
        self._cache: Dict[Tuple, Tuple] = {}
        functools.update_wrapper(self, fn)

    def _compile(self, args):
        shape = tuple(args[0].shape)
        tr = _Trace(shape)
        syms = [tr.input(a) for a in args]
        res = self.fn(*syms)
        outs = list(res) if isinstance(res, (tuple, list)) else [res]
        if not 1 <= len(outs) <= _MAX_OUT:
            raise ValueError(f"a fused function returns 1 to {_MAX_OUT} arrays")
        refs = []
        for o in outs:
            if not isinstance(o, _Sym):
                raise TypeError("a fused function must return traced arrays")
            refs.append(o._ref)
        n_in = len(tr.inputs)
        digest = hashlib.sha1("\n".join(tr.lines + refs).encode()).hexdigest()[:16]
        name = f"vkc_fused_{digest}"
        src = _source(name, tr, refs, n_in)
        gpu = args[0]._gpu
        k = C.c_void_p()
        check(lib.vkc_jit_compile(gpu._dev.h, src.encode(), name.encode(), C.byref(k)))
        # which call argument feeds each kernel input slot
        slots = [next(i for i, a in enumerate(args) if a is arr) for arr in tr.inputs]
        return k, slots, len(refs), src

    def __call__(self, *args: Array):
        if not args or not all(isinstance(a, Array) for a in args):
            raise TypeError("fused functions take vulkpy_gb300 Arrays")
        key = tuple((tuple(a.shape), a._gpu._idx) for a in args) + \
            tuple(tuple(i for i, b in enumerate(args) if b is a) for a in args)
        ent = self._cache.get(key)
        if ent is None:
            ent = self._cache[key] = self._compile(args)
        k, slots, n_out, _ = ent
        gpu = args[0]._gpu
        outs = [Array(gpu, shape=args[0].shape) for _ in range(n_out)]
        ins = (C.c_void_p * _MAX_IN)(*[args[s]._dptr() for s in slots])
        optr = (C.c_void_p * _MAX_OUT)(*[o._buf.ptr for o in outs])
        check(lib.vkc_jit_launch(gpu._dev.h, k, ins, len(slots), optr, n_out, args[0].size))
        for o in outs:
            o._written()
        return outs[0] if n_out == 1 else tuple(outs)

    def source(self, *args: Array) -> str:
        """The generated CUDA source for these argument shapes."""
        return self._compile(args)[3]


def fuse(fn: Callable) -> FusedFunction:
    """Decorator: compile an elementwise function of Arrays into one kernel."""
    return FusedFunction(fn)
