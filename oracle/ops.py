"""
numpy-level oracle functions (test infrastructure; see oracle/__init__.py).

Every function takes and returns numpy arrays and runs the C restatement in
oracle/vkoracle.c, except the ``truth_*`` helpers which compute in float64
for error bounds.
"""
from __future__ import annotations

import numpy as np

from . import lib

ADD, SUB, MUL, DIV, POW, MAX, MIN, RSUB, RDIV, RPOW = range(10)
UNARY = ["abs", "sign", "sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh", "tanh",
         "asinh", "acosh", "atanh", "exp", "log", "exp2", "log2", "sqrt", "invsqrt"]
SUM, PROD, MAXIMUM, MINIMUM = range(4)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


# ------------------------------------------------------------------ PRNG
class Xoshiro128pp:
    """Restatement of PRNG::Xoshiro128pp (vulkpy/_vkarray.cc:589-717)."""

    def __init__(self, seed: int, size: int = 64):
        self.size = int(size)
        self.state = np.zeros(4 * self.size, dtype=np.uint32)
        lib().xo_seed(int(seed), self.size, _p(self.state))

    def u32(self, n: int) -> np.ndarray:
        out = np.empty(int(n), dtype=np.uint32)
        lib().xo_generate(_p(self.state), self.size, _p(out), int(n), 0)
        return out

    def f32(self, n: int) -> np.ndarray:
        out = np.empty(int(n), dtype=np.float32)
        lib().xo_generate(_p(self.state), self.size, _p(out), int(n), 1)
        return out

    def normal(self, n: int, mean: float = 0.0, stddev: float = 1.0) -> np.ndarray:
        """random.py:60-124: n uniforms (n+1 for odd n), Box-Muller on pairs."""
        n = int(n)
        m = n if n % 2 == 0 else n + 1
        u = self.f32(m)
        out = np.empty(n, dtype=np.float32)
        lib().box_muller(_p(u), _p(out), n, np.float32(mean), np.float32(stddev))
        return out

    def randrange(self, n: int, low: int, high: int) -> np.ndarray:
        """random.py:126-186 with prng_randrange.comp (high exclusive)."""
        if low == 0 and high == 2 ** 32:
            return self.u32(n)
        u = self.f32(n)
        out = np.empty(int(n), dtype=np.uint32)
        lib().randrange(_p(u), _p(out), int(n), int(low), int(high) - 1)
        return out

    def permutation(self, n: int) -> np.ndarray:
        """Four keys from the u32 stream, then the keyed Feistel permutation
        (vkoracle.c ``permutation``)."""
        out = np.empty(int(n), dtype=np.uint32)
        if n:   # an empty permutation draws nothing
            key = self.u32(4)
            lib().permutation(_p(key), _p(out), int(n))
        return out


# ------------------------------------------------------------ elementwise
def binary(op: int, a, b) -> np.ndarray:
    a, b = _f32(a), _f32(b)
    assert a.shape == b.shape
    c = np.empty_like(a)
    lib().ew_binary(op, _p(a), _p(b), _p(c), a.size)
    return c


def scalar(op: int, a, s: float) -> np.ndarray:
    a = _f32(a)
    c = np.empty_like(a)
    lib().ew_scalar(op, _p(a), np.float32(s), _p(c), a.size)
    return c


def unary(name: str, a) -> np.ndarray:
    a = _f32(a)
    c = np.empty_like(a)
    lib().ew_unary(UNARY.index(name), _p(a), _p(c), a.size)
    return c


def bcast(op: int, a, b) -> np.ndarray:
    """add_broadcast.comp:25-45 index math over numpy-broadcast shapes."""
    a, b = _f32(a), _f32(b)
    shape = np.broadcast_shapes(a.shape, b.shape)
    nd = len(shape)
    sa = np.array((1,) * (nd - a.ndim) + a.shape, dtype=np.int64)
    sb = np.array((1,) * (nd - b.ndim) + b.shape, dtype=np.int64)
    sc = np.array(shape, dtype=np.int64)
    c = np.empty(shape, dtype=np.float32)
    lib().bcast_binary(op, _p(a), _p(sa), _p(b), _p(sb), _p(c), _p(sc), nd)
    return c


def clamp(a, lo, hi) -> np.ndarray:
    """clamp*.comp: min(max(a, lo), hi) after broadcasting."""
    a = _f32(a)
    return np.fmin(np.fmax(a, np.float32(lo) if np.ndim(lo) == 0 else _f32(lo)),
                   np.float32(hi) if np.ndim(hi) == 0 else _f32(hi)).astype(np.float32)


# ------------------------------------------------------------ reductions
def reduce_axis(op: int, a, axis) -> np.ndarray:
    """*_axis.comp serial loops, one axis at a time in descending order
    (vkarray.py:1194-1222)."""
    t = _f32(a)
    axes = sorted({int(x) % t.ndim for x in np.atleast_1d(axis)}, reverse=True)
    for ax in axes:
        prev = int(np.prod(t.shape[:ax]))
        n = t.shape[ax]
        post = int(np.prod(t.shape[ax + 1:]))
        out = np.empty(t.shape[:ax] + t.shape[ax + 1:], dtype=np.float32)
        lib().reduce_axis(op, _p(t), prev, n, post, _p(out))
        t = out
    return t


def reduce_all(op: int, a) -> np.float32:
    a = _f32(a)
    return np.float32(lib().reduce_all(op, _p(a), a.size))


# ------------------------------------------------------------ matmul, gather
def matmul(a, b) -> np.ndarray:
    """matmul.comp:23-33 (serial K loop per output)."""
    a, b = _f32(a), _f32(b)
    M = int(np.prod(a.shape[:-1])) if a.ndim > 1 else 1
    K = a.shape[-1]
    N = int(np.prod(b.shape[1:])) if b.ndim > 1 else 1
    c = np.empty(a.shape[:-1] + b.shape[1:], dtype=np.float32)
    lib().matmul(_p(a), _p(b), _p(c), M, K, N)
    return c


def gather(a, idx) -> np.ndarray:
    a = _f32(a)
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    c = np.empty(idx.shape, dtype=np.float32)
    lib().gather(_p(a), a.size, _p(idx), idx.size, _p(c))
    return c


def gather_axis(a, idx, axis: int) -> np.ndarray:
    """gather_axis.comp layout: [idx..., prev..., post...]."""
    a = _f32(a)
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    prev = int(np.prod(a.shape[:axis]))
    post = int(np.prod(a.shape[axis + 1:]))
    c = np.empty(idx.shape + a.shape[:axis] + a.shape[axis + 1:], dtype=np.float32)
    lib().gather_axis(_p(a), prev, a.shape[axis], post, _p(idx), idx.size, _p(c))
    return c


# ------------------------------------------------------------ float64 truth
def ulp_distance(x, y) -> np.ndarray:
    """|x - y| in units of float32 ulp of y (y rounded to float32)."""
    x = np.asarray(x, dtype=np.float32)
    y32 = np.asarray(y, dtype=np.float64).astype(np.float32)
    spacing = np.spacing(np.abs(y32)).astype(np.float64)
    spacing = np.where(spacing == 0, np.finfo(np.float32).smallest_subnormal, spacing)
    return np.abs(x.astype(np.float64) - np.asarray(y, dtype=np.float64)) / spacing


def rel_fro(x, ref) -> float:
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.linalg.norm(np.asarray(x, dtype=np.float64) - ref) / np.linalg.norm(ref))
