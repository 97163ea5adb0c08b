"""Matrix-vector products (M == 1 or N == 1 GEMMs, 1-D operands of `@`):
fp32 GEMV for every matmul precision, checked against float64."""
import ctypes as C

import numpy as np
import pytest

from oracle.ops import rel_fro

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
@pytest.mark.parametrize("k,n", [(4096, 4096), (1, 7), (1000, 3), (33, 2050), (8192, 1)])
def test_vector_at_matrix(gpu, vk, prec, k, n):
    rng = np.random.default_rng(k + n)
    v = rng.standard_normal(k).astype(np.float32)
    B = rng.standard_normal((k, n)).astype(np.float32)
    got = np.asarray(vk.vkarray.matmul(vk.Array(gpu, data=v), vk.Array(gpu, data=B), precision=prec))
    assert got.shape == (n,)
    _check_sums(got, v[None, :], B)
    assert gpu.check_errors() == 0


def _check_sums(got, A, B):
    """fp32 summation error against float64, per output relative to the sum
    of |terms| (the scale of rounding error; a single dot product of N(0,1)
    values cancels, so its relative error alone is no bound): <= 2e-6, i.e.
    ~34 ulp of that scale for K up to 8192."""
    A64, B64 = A.astype(np.float64), B.astype(np.float64)
    exact = (A64 @ B64).reshape(got.shape)
    scale = (np.abs(A64) @ np.abs(B64)).reshape(got.shape)
    assert np.all(np.abs(got - exact) <= 2e-6 * scale + 1e-30), np.max(np.abs(got - exact) / scale)


@pytest.mark.parametrize("m,k", [(4096, 4096), (7, 1), (3, 1000), (2050, 33)])
def test_matrix_at_vector(gpu, vk, m, k):
    rng = np.random.default_rng(m * 3 + k)
    A = rng.standard_normal((m, k)).astype(np.float32)
    v = rng.standard_normal(k).astype(np.float32)
    got = np.asarray(vk.Array(gpu, data=A) @ vk.Array(gpu, data=v))
    assert got.shape == (m,)
    _check_sums(got, A, v[:, None])


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("M,N", [(1, 300), (300, 1), (1, 1)])
def test_gemv_transposes_alpha_beta(gpu, vk, ta, tb, M, N):
    """vkc_gemm with a unit dimension, both operand orientations, alpha and beta."""
    from vulkpy_gb300 import _lib
    rng = np.random.default_rng(ta * 2 + tb + M)
    K = 517
    A = rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
    C0 = rng.standard_normal((M, N)).astype(np.float32)
    a, b, c = vk.Array(gpu, data=A), vk.Array(gpu, data=B), vk.Array(gpu, data=C0)
    st = _lib.lib.vkc_gemm(gpu.handle, _lib.MM_FP32, ta, tb, M, N, K, C.c_float(0.5), a._dptr(), A.shape[1],
                           b._dptr(), B.shape[1], C.c_float(2.0), c._dptr(), N)
    assert st == 0, _lib.last_error()
    c._written()
    exp = 0.5 * ((A.T if ta else A).astype(np.float64) @ (B.T if tb else B)) + 2.0 * C0
    assert rel_fro(np.asarray(c), exp) < 1e-6


@pytest.mark.parametrize("prec", ["fp32", "bf16x3"])
def test_dense_batch_one(gpu, vk, prec):
    """A Dense layer on one sample: forward (bias + ReLU epilogue) and the
    backward products are vector products."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal((1, 300)).astype(np.float32)
    W = (rng.standard_normal((64, 300)) * 0.1).astype(np.float32)
    bvec = rng.standard_normal(64).astype(np.float32)
    dy = rng.standard_normal((1, 64)).astype(np.float32)
    old = gpu.matmul_precision
    gpu.matmul_precision = prec
    try:
        d = vk.nn.Dense(gpu, 300, 64, w_init=lambda g, s: vk.Array(g, data=W),
                        b_init=lambda g, s: vk.Array(g, data=bvec))
        y = np.asarray(d(vk.Array(gpu, data=x)))
        dx = np.asarray(d.backward(vk.Array(gpu, data=dy)))
        dW = np.asarray(d.w.grad)
        db = np.asarray(d.b.grad)
    finally:
        gpu.matmul_precision = old
    x64 = x.astype(np.float64)
    assert rel_fro(y, x64 @ W.T.astype(np.float64) + bvec) < 1e-6
    assert rel_fro(dx, dy.astype(np.float64) @ W.astype(np.float64)) < 1e-6
    # dW = dy^T x is 64 x 300 with K = 1: a tiled GEMM in the requested precision
    assert rel_fro(dW, dy.astype(np.float64).T @ x64) < (1e-6 if prec == "fp32" else 1e-5)
    np.testing.assert_allclose(db, dy[0], rtol=1e-6)
