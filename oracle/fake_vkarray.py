"""
numpy stand-in for vulkpy's native module ``_vkarray`` (TEST INFRASTRUCTURE).

vulkpy's Python layer (vkarray.py, random.py, nn/) talks to the GPU only
through the pybind11 module ``_vkarray`` (vulkpy/_vkarray.cc:756-898):
buffers with the buffer protocol, ``GPU.submit(spv, local_size, buffers,
DataShape, Params, jobs)`` and ``Xoshiro128pp``.  This module provides the
same names, and ``submit`` runs a numpy/C restatement of the named shader's
``main()`` over the dispatched invocation range, immediately.  Buffers start
filled with NaN so that reading memory the reference never writes shows up.

``load_reference(path)`` imports the reference package from its source tree
with this module installed as ``vulkpy._vkarray`` (and a minimal ``wblog``),
so the reference's own Python code -- and its own unittest suites -- run on
the CPU.  Used to generate and pin tests/golden; never by the product.
"""
from __future__ import annotations

import importlib
import importlib.util
import logging
import os
import secrets
import sys
import types

import numpy as np

from . import ops as O

f32 = np.float32


# ------------------------------------------------------------------ buffers
class _Buffer:
    def __init__(self, n: int, dtype, data=None):
        if data is not None:
            self._a = np.array(np.asarray(data).reshape(-1), dtype=dtype)
        else:
            self._a = np.full(int(n), np.nan if dtype == np.float32 else 0xDEADBEEF, dtype=dtype)

    def __array__(self, dtype=None, copy=None):
        return self._a

    def flat(self) -> np.ndarray:
        return self._a.reshape(-1)

    def size(self) -> int:
        return self._a.size

    def info(self):
        return self

    def range(self):
        return self


Buffer = _Buffer
Shape = _Buffer


class Job:
    def wait(self, timeout_ns=None):
        return None


class DataShape:
    def __init__(self, x, y, z):
        self.x, self.y, self.z = int(x), int(y), int(z)


def _params(name, *fields):
    def __init__(self, *args):
        if len(args) != len(fields):
            raise TypeError(f"{name} takes {len(fields)} arguments")
        for f, v in zip(fields, args):
            setattr(self, f, v)
    return type(name, (), {"__init__": __init__, "_fields": fields})


VectorParams = _params("VectorParams", "size")
MultiVector2Params = _params("MultiVector2Params", "size0", "size1")
VectorScalarParams = _params("VectorScalarParams", "size", "scalar")
VectorScalar2Params = _params("VectorScalar2Params", "size", "scalar0", "scalar1")
MatMulParams = _params("MatMulParams", "rowA", "contractSize", "columnB")
AxisReductionParams = _params("AxisReductionParams", "prev_prod", "axis_size", "post_prod")
BroadcastParams = _params("BroadcastParams", "size0", "size1", "ndim")
Multi3BroadcastParams = _params("Multi3BroadcastParams", "size0", "size1", "size2", "ndim")
BatchAffineParams = _params("BatchAffineParams", "batch_size", "input_size", "output_size")
VectorRangeParams = _params("VectorRangeParams", "size", "low", "high")
AxisGatherParams = _params("AxisGatherParams", "prev_prod", "post_prod", "axis_size", "index_size")


# ------------------------------------------------------------------ shaders
_BIN = {"add": O.ADD, "sub": O.SUB, "mul": O.MUL, "div": O.DIV, "pow": O.POW, "max": O.MAX, "min": O.MIN}
_RSCALAR = {"rsub_scalar": O.RSUB, "rdiv_scalar": O.RDIV, "rpow_scalar": O.RPOW}


def _binop(op, a, b):
    a = np.asarray(a, dtype=f32)
    b = np.asarray(b, dtype=f32)
    with np.errstate(all="ignore"):
        if op == O.ADD: return (a + b).astype(f32)
        if op == O.SUB: return (a - b).astype(f32)
        if op == O.MUL: return (a * b).astype(f32)
        if op == O.DIV: return (a / b).astype(f32)
        if op == O.POW:
            if np.ndim(b) == 0 and b == 2.0:
                return (a * a).astype(f32)
            return np.power(a, b).astype(f32)
        if op == O.MAX: return np.fmax(a, b).astype(f32)
        if op == O.MIN: return np.fmin(a, b).astype(f32)
    raise ValueError(op)


def _unop(name, a):
    a = np.asarray(a, dtype=f32)
    with np.errstate(all="ignore"):
        if name == "invsqrt":
            return (f32(1) / np.sqrt(a)).astype(f32)
        fn = {"abs": np.abs, "sign": np.sign, "sin": np.sin, "cos": np.cos, "tan": np.tan, "asin": np.arcsin,
              "acos": np.arccos, "atan": np.arctan, "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh,
              "asinh": np.arcsinh, "acosh": np.arccosh, "atanh": np.arctanh, "exp": np.exp, "log": np.log,
              "exp2": np.exp2, "log2": np.log2, "sqrt": np.sqrt}[name]
        return fn(a).astype(f32)


def _bcast_index3(ci, shapes, sizes, ndim):
    """add_broadcast.comp:25-45 for a vector of output indices ci."""
    size = np.array(sizes, dtype=np.int64)
    ab = np.zeros((2, ci.size), dtype=np.int64)
    rem = ci.astype(np.int64)
    for dim in range(ndim):
        s = np.array([shapes[dim], shapes[dim + ndim], shapes[dim + 2 * ndim]], dtype=np.int64)
        size = size // s
        d = rem // size[2]
        ab[0] += size[0] * np.minimum(d, s[0] - 1)
        ab[1] += size[1] * np.minimum(d, s[1] - 1)
        rem = rem % size[2]
    return ab


def _bcast_views(shapes, ndim, a, b):
    """When every operand dim is 1 or the output's, add_broadcast.comp's
    index sum_k stride_k * min(d_k, s_k - 1) is exactly numpy broadcasting:
    return the operands as broadcast views of the output shape (None when
    the shapes need the shader's clamping)."""
    sa = [int(x) for x in shapes[0:ndim]]
    sb = [int(x) for x in shapes[ndim:2 * ndim]]
    sc = [int(x) for x in shapes[2 * ndim:3 * ndim]]
    for s in (sa, sb):
        if any(x not in (1, c) for x, c in zip(s, sc)):
            return None
    na, nb = int(np.prod(sa)), int(np.prod(sb))
    if a.size < na or b.size < nb:
        return None
    return np.broadcast_to(a[:na].reshape(sa), sc), np.broadcast_to(b[:nb].reshape(sb), sc)


def _bcast_index2(ai, shapes, sizes, ndim):
    """iadd_broadcast.comp:22-41 (index into b for every element of a)."""
    size = np.array(sizes, dtype=np.int64)
    bi = np.zeros(ai.size, dtype=np.int64)
    rem = ai.astype(np.int64)
    for dim in range(ndim):
        s = np.array([shapes[dim], shapes[dim + ndim]], dtype=np.int64)
        size = size // s
        d = rem // size[0]
        bi += size[1] * np.minimum(d, s[1] - 1)
        rem = rem % size[0]
    return bi


def _run(name: str, bufs, ds: DataShape, p):
    B = [b.flat() for b in bufs]
    if name in _BIN:                          # c = a op b
        n = min(p.size, ds.x)
        B[2][:n] = _binop(_BIN[name], B[0][:n], B[1][:n])
        return
    if name[0] == "i" and name[1:] in _BIN:   # a = a op b
        n = min(p.size, ds.x)
        B[0][:n] = _binop(_BIN[name[1:]], B[0][:n], B[1][:n])
        return
    if name.endswith("_scalar"):
        base = name[:-7]
        n = min(p.size, ds.x)
        s = f32(p.scalar)
        if name in _RSCALAR:
            op = {"rsub_scalar": O.SUB, "rdiv_scalar": O.DIV, "rpow_scalar": O.POW}[name]
            B[1][:n] = _binop(op, s, B[0][:n]) if op != O.POW else np.power(s, B[0][:n]).astype(f32)
        elif base in _BIN:
            B[1][:n] = _binop(_BIN[base], B[0][:n], s)
        elif base[0] == "i" and base[1:] in _BIN:
            B[0][:n] = _binop(_BIN[base[1:]], B[0][:n], s)
        else:
            raise NotImplementedError(name)
        return
    if name.endswith("_broadcast"):
        base = name[:-10]
        if base in _BIN:                       # Multi3BroadcastParams
            n = min(p.size2, ds.x)
            views = _bcast_views(B[3], p.ndim, B[0], B[1]) if n == p.size2 else None
            if views is not None:
                B[2][:n] = _binop(_BIN[base], views[0], views[1]).reshape(-1)
                return
            ci = np.arange(n)
            ab = _bcast_index3(ci, B[3], (p.size0, p.size1, p.size2), p.ndim)
            B[2][:n] = _binop(_BIN[base], B[0][ab[0]], B[1][ab[1]])
            return
        if base[0] == "i" and base[1:] in _BIN:  # BroadcastParams
            n = min(p.size0, ds.x)
            ai = np.arange(n)
            bi = _bcast_index2(ai, B[2], (p.size0, p.size1), p.ndim)
            B[0][:n] = _binop(_BIN[base[1:]], B[0][:n], B[1][bi])
            return
    if name in O.UNARY:
        n = min(p.size, ds.x)
        B[1][:n] = _unop(name, B[0][:n])
        return
    if name[0] == "i" and name[1:] in O.UNARY:
        n = min(p.size, ds.x)
        B[0][:n] = _unop(name[1:], B[0][:n])
        return
    if name.startswith("clamp") or name.startswith("iclamp"):
        n = min(p.size, ds.x)
        kind = name.split("_")[1] if "_" in name else "vv"
        inplace = name.startswith("i")
        a = B[0][:n]
        if kind == "vv":
            lo, hi, out = B[1][:n], B[2][:n], (B[0] if inplace else B[3])
        elif kind == "sv":
            lo, hi, out = f32(p.scalar), B[1][:n], (B[0] if inplace else B[2])
        elif kind == "vs":
            lo, hi, out = B[1][:n], f32(p.scalar), (B[0] if inplace else B[2])
        else:
            lo, hi, out = f32(p.scalar0), f32(p.scalar1), (B[0] if inplace else B[1])
        out[:n] = np.fmin(np.fmax(a, lo), hi)
        return
    for red, op in (("sum", O.SUM), ("prod", O.PROD), ("maximum", O.MAXIMUM), ("minimum", O.MINIMUM)):
        if name == red:                        # strided partials, sum.comp:18-30
            sa, sb = p.size0, p.size1
            for i in range(min(ds.x, sb)):
                col = B[0][i:sa:sb]
                if op == O.SUM:
                    acc = f32(0)
                    for v in col: acc = f32(acc + v)
                elif op == O.PROD:
                    acc = f32(1)
                    for v in col: acc = f32(acc * v)
                elif op == O.MAXIMUM:
                    acc = B[0][i]
                    for v in col: acc = np.fmax(acc, v)
                else:
                    acc = B[0][i]
                    for v in col: acc = np.fmin(acc, v)
                B[1][i] = acc
            return
        if name == red + "_axis":
            prev, n, post = p.prev_prod, p.axis_size, p.post_prod
            a = np.ascontiguousarray(B[0][:prev * n * post]).reshape(prev, n, post)
            B[1][:prev * post] = O.reduce_axis(op, a, 1).reshape(-1)
            return
        if name == red + "_axis_rebroadcast":
            prev, n, post = p.prev_prod, p.axis_size, p.post_prod
            a = np.ascontiguousarray(B[0][:prev * n * post]).reshape(prev, n, post)
            r = O.reduce_axis(op, a, 1)
            B[1][:prev * n * post] = np.broadcast_to(r[:, None, :], (prev, n, post)).reshape(-1)
            return
    if name == "broadcast":                    # broadcast.comp:25-44
        n = min(p.size1, ds.x)
        i_tmp = np.arange(n, dtype=np.int64)
        j = np.zeros(n, dtype=np.int64)
        sa, sb = p.size0, p.size1
        for dim in range(p.ndim):
            sa //= int(B[2][dim])
            sb //= int(B[3][dim])
            d = np.minimum(i_tmp // sb, int(B[2][dim]) - 1)
            j += d * sa
            i_tmp = i_tmp % sb
        B[1][:n] = B[0][j]
        return
    if name == "gather":
        n = min(p.size, ds.x)
        B[2][:n] = B[0][B[1][:n].astype(np.int64)]
        return
    if name == "gather_axis":                  # gather_axis.comp:24-43
        prev, post, axis, ni = p.prev_prod, p.post_prod, p.axis_size, p.index_size
        a = B[0][:prev * axis * post].reshape(prev, axis, post)
        bk = np.clip(B[1][:ni].astype(np.int64), 0, axis)
        B[2][:ni * prev * post] = a[:, bk, :].transpose(1, 0, 2).reshape(-1)
        return
    if name == "matmul":
        M, K, N = p.rowA, p.contractSize, p.columnB
        B[2][:M * N] = O.matmul(B[0][:M * K].reshape(M, K), B[1][:K * N].reshape(K, N)).reshape(-1)
        return
    if name == "batch_affine":                 # batch_affine.comp:25-39
        nb, ni, no = p.batch_size, p.input_size, p.output_size
        w = B[0][:no * ni].reshape(no, ni)
        x = B[2][:nb * ni].reshape(nb, ni)
        y = O.matmul(x, np.ascontiguousarray(w.T))
        B[3][:nb * no] = (y + B[1][:no][None, :]).astype(f32).reshape(-1)
        return
    if name == "nn_cross_entropy":
        n = min(p.size, ds.x)
        with np.errstate(all="ignore"):
            B[2][:n] = (-B[1][:n] * np.log(B[0][:n] + f32(1e-8))).astype(f32)
        return
    if name == "nn_cross_entropy_backward":
        n = min(p.size, ds.x)
        with np.errstate(all="ignore"):
            B[2][:n] = (-B[1][:n] / (B[0][:n] + f32(1e-8))).astype(f32)
        return
    if name in ("prng_box_muller", "prng_ibox_muller"):
        size = p.size
        j = 2 * np.arange(ds.x)                 # whole workgroups of the n//2 dispatch
        j = j[j < size]                         # prng_box_muller.comp:22
        k = j + 1
        src = B[0]
        dst = B[0] if name == "prng_ibox_muller" else B[1]
        u0 = src[j].astype(f32)
        u1 = src[k].astype(f32)
        with np.errstate(all="ignore"):
            r = np.sqrt(f32(-2) * np.log(f32(1) - u0)).astype(f32) * f32(p.scalar1)
            angle = f32(6.28318530718) * u1
            z0 = (f32(p.scalar0) + r * np.sin(angle)).astype(f32)
            z1 = (f32(p.scalar0) + r * np.cos(angle)).astype(f32)
        ok0 = j < size
        dst[j[ok0]] = z0[ok0]
        ok1 = k < size
        dst[k[ok1]] = z1[ok1]
        return
    if name == "prng_randrange":
        n = min(p.size, ds.x)
        rng = np.uint32(np.uint32(p.high) - np.uint32(p.low) + np.uint32(1))
        with np.errstate(all="ignore"):
            B[1][:n] = (np.uint32(p.low) + (f32(rng) * B[0][:n]).astype(np.uint32)).astype(np.uint32)
        return
    raise NotImplementedError(f"shader {name} is not restated in the oracle")


class GPU:
    def __init__(self, idx: int, priority: float):
        self.idx = idx

    def toBuffer(self, data):
        return _Buffer(0, np.float32, data)

    def createBuffer(self, n):
        return _Buffer(n, np.float32)

    def toU32Buffer(self, data):
        return _Buffer(0, np.uint32, data)

    def createU32Buffer(self, n):
        return _Buffer(n, np.uint32)

    def submit(self, spv, x, y, z, infos, shape, params, jobs):
        name = os.path.basename(str(spv))
        if name.endswith(".spv"):
            name = name[:-4]
        # Vulkan runs whole workgroups: ceil(DataShape / local_size) groups
        # (_vkarray.cc:333-335); each shader bounds-checks against its params.
        ds = DataShape(-(-shape.x // x) * x, -(-shape.y // y) * y, -(-shape.z // z) * z)
        _run(name, infos, ds, params)
        return Job()

    def wait(self):
        return None

    def flush(self, ranges):
        return None

    def canSubgroupArithmetic(self):
        return False


def createGPU(idx, priority):
    return GPU(idx, priority)


class Xoshiro128pp:
    """PRNG::Xoshiro128pp (vulkpy/_vkarray.cc:589-717) over the C restatement."""

    def __init__(self, gpu, spv_uint32, spv_float, size, seed=None):
        if seed is None:
            seed = secrets.randbits(32)
        self._rng = O.Xoshiro128pp(int(seed), int(size))

    def random_uint32(self, n, info):
        info.flat()[:n] = self._rng.u32(n)
        return Job()

    def random_float(self, n, info):
        info.flat()[:n] = self._rng.f32(n)
        return Job()


# ------------------------------------------------------------------ loader
def load_reference(root: str, name: str = "vulkpy"):
    """Import the reference package at ``root/vulkpy`` with this fake as its
    native module.  Returns the package module."""
    if "wblog" not in sys.modules:
        wb = types.ModuleType("wblog")
        wb.getLogger = lambda *a, **k: logging.getLogger("vulkpy-reference")
        wb.start_logging = lambda *a, **k: None
        sys.modules["wblog"] = wb
    pkg_dir = os.path.join(root, "vulkpy")
    fake = sys.modules[__name__]
    sys.modules[f"{name}._vkarray"] = fake
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod
