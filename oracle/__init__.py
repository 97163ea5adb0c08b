"""
Oracle -- CPU restatement of vulkpy's algorithms.  TEST INFRASTRUCTURE ONLY.

This package is the checker for the CUDA path and the timed CPU baseline.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it; the product (``vulkpy_gb300``) never does.

Contents
--------
* ``vkoracle.c`` (built to ``_build/libvkoracle.so`` by :func:`build`):
  plain-C restatement of the reference's shader loops and of its PRNG,
  bit-exact for the integer work (see the header of that file for the
  reference file:line each function follows).
* :mod:`oracle.ops` -- numpy wrappers over the C library plus float64
  "truth" helpers used for error bounds.
* :mod:`oracle.fake_vkarray` -- a numpy stand-in for vulkpy's native module
  ``_vkarray`` that lets the reference's own Python (vkarray.py, random.py,
  nn/) run on the CPU where the reference source is available; used only
  to generate and pin the golden fixtures in ``tests/golden``.

Parity pins: the PRNG restatement has no golden values in the reference's
tests (vulkpy's test_random.py checks ranges and reproducibility only), so
the raw stream is pinned by the source restatement; the shader restatement
is pinned by running the reference's own unittest suites against
``fake_vkarray`` (tests/test_oracle_reference.py).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "vkoracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "libvkoracle.so"

_CFLAGS = ["-O2", "-fopenmp", "-fPIC", "-shared", "-fvisibility=hidden", "-ffp-contract=off", "-std=c11"]


def build(force: bool = False) -> Path:
    """Compile vkoracle.c with gcc (OpenMP, no FMA contraction)."""
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([cc, *_CFLAGS, "-o", str(tmp), str(SRC), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        vp, u64, u32, i32, f32, i64 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, C.c_float, C.c_int64
        sig = {
            "xo_seed": ([u64, u32, vp], None),
            "xo_generate": ([vp, u32, vp, u64, i32], None),
            "box_muller": ([vp, vp, u64, f32, f32], None),
            "randrange": ([vp, vp, u64, u32, u32], None),
            "ew_binary": ([i32, vp, vp, vp, u64], None),
            "ew_scalar": ([i32, vp, f32, vp, u64], None),
            "ew_unary": ([i32, vp, vp, u64], None),
            "bcast_binary": ([i32, vp, vp, vp, vp, vp, vp, i32], None),
            "reduce_axis": ([i32, vp, u64, u64, u64, vp], None),
            "reduce_all": ([i32, vp, u64], f32),
            "matmul": ([vp, vp, vp, i64, i64, i64], None),
            "gather": ([vp, u64, vp, u64, vp], None),
            "gather_axis": ([vp, u64, u64, u64, vp, u64, vp], None),
            "permutation": ([vp, vp, u64], None),
            "oracle_threads": ([], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib
