"""The fused-kernel code generator (CPU): a traced chain becomes CUDA C
that compiles for sm_103a; scalar constants are exact float32 literals."""
import os
import shutil
import subprocess

import numpy as np
import pytest


class _FakeArray:
    def __init__(self, shape):
        self.shape = shape


def _trace(fn, n_args=2):
    from vulkpy_gb300 import fusion as F
    tr = F._Trace((16,))
    syms = [tr.input(_FakeArray((16,))) for _ in range(n_args)]
    res = fn(*syms)
    outs = list(res) if isinstance(res, tuple) else [res]
    return F._source("vkc_fused_test", tr, [o._ref for o in outs], len(tr.inputs)), tr


def test_literals_are_exact():
    from vulkpy_gb300.fusion import _lit
    for v in (1.0001, 0.1, -2.5, 1e-30, 3.4e38):
        lit = _lit(v)
        assert float.fromhex(lit[:-1]) == float(np.float32(v))
    assert "__int_as_float" in _lit(float("inf"))


def test_chain_source_compiles_for_sm103a(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    import bench
    src, tr = _trace(bench.chain32)
    assert src.count("const float t") == 32
    f = tmp_path / "k.cu"
    f.write_text(src)
    r = subprocess.run([nvcc, "-arch=sm_103a", "-fmad=false", "-cubin", "-o", str(tmp_path / "k.cubin"), str(f)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_square_and_reversed_ops():
    src, _ = _trace(lambda x, y: ((2.0 - x) ** 2.0, 3.0 / y, 1.5 ** x))
    assert "t0 * t0" in src and "/ x[1]" in src and "powf(0x1.8" in src
