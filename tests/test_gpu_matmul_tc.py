"""Tensor-core (tcgen05) matmul: bf16 and split-bf16x3 against float64.

Bounds (relative Frobenius error vs float64, N(0,1) inputs):
  * bf16:    operands rounded to 8 significant bits -> ~3e-3; bound 8e-3.
  * bf16x3:  hi/lo split keeps ~16 bits per operand -> a few 1e-6; bound 1e-5
             (the accuracy target for the split method).
The device error word must stay clear (no pipeline wait expired)."""
import numpy as np
import pytest

from oracle.ops import rel_fro

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128, 64), (128, 256, 128), (256, 512, 320), (129, 257, 100), (1, 300, 7), (300, 1, 513),
          (1000, 1000, 1000), (64, 2048, 8), (256, 384, 4096), (512, 512, 8192)]


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


@pytest.mark.parametrize("m,n,k", SHAPES)
@pytest.mark.parametrize("prec,bound", [("bf16", 8e-3), ("bf16x3", 1e-5)])
def test_tc_matmul_accuracy(gpu, vk, m, n, k, prec, bound):
    gpu.check_errors()
    rng = np.random.default_rng(m * 7 + n * 13 + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((k, n)).astype(np.float32)
    got = np.asarray(vk.vkarray.matmul(vk.Array(gpu, data=a), vk.Array(gpu, data=b), precision=prec))
    assert gpu.check_errors() == 0
    err = rel_fro(got, a.astype(np.float64) @ b.astype(np.float64))
    assert err < bound, (prec, m, n, k, err)


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_tc_gemm_transposes_alpha_beta(gpu, vk, ta, tb):
    """vkc_gemm through the C ABI with transposed operands, alpha and beta."""
    import ctypes as C
    from vulkpy_gb300 import _lib
    rng = np.random.default_rng(ta * 2 + tb)
    M, N, K = 200, 136, 72
    A = rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
    C0 = rng.standard_normal((M, N)).astype(np.float32)
    a, b, c = vk.Array(gpu, data=A), vk.Array(gpu, data=B), vk.Array(gpu, data=C0)
    st = _lib.lib.vkc_gemm(gpu.handle, _lib.MM_BF16X3, ta, tb, M, N, K, C.c_float(0.5), a._dptr(), A.shape[1],
                           b._dptr(), B.shape[1], C.c_float(2.0), c._dptr(), N)
    assert st == 0, _lib.last_error()
    c._written()
    opA = A.T if ta else A
    opB = B.T if tb else B
    exp = 0.5 * (opA.astype(np.float64) @ opB) + 2.0 * C0
    assert rel_fro(np.asarray(c), exp) < 1e-5
    assert gpu.check_errors() == 0


def test_dense_layer_on_tensor_cores(gpu, vk):
    rng = np.random.default_rng(9)
    x = rng.standard_normal((256, 784)).astype(np.float32)
    W = (rng.standard_normal((1024, 784)) * 0.05).astype(np.float32)
    bvec = rng.standard_normal(1024).astype(np.float32)
    old = gpu.matmul_precision
    gpu.matmul_precision = "bf16x3"
    try:
        d = vk.nn.Dense(gpu, 784, 1024, w_init=lambda g, s: vk.Array(g, data=W),
                        b_init=lambda g, s: vk.Array(g, data=bvec))
        y = np.asarray(d(vk.Array(gpu, data=x)))
        dy = rng.standard_normal((256, 1024)).astype(np.float32)
        dx = np.asarray(d.backward(vk.Array(gpu, data=dy)))
        dW = np.asarray(d.w.grad)
    finally:
        gpu.matmul_precision = old
    x64 = x.astype(np.float64)
    assert rel_fro(y, x64 @ W.T.astype(np.float64) + bvec) < 1e-5
    assert rel_fro(dx, dy.astype(np.float64) @ W.astype(np.float64)) < 1e-5
    assert rel_fro(dW, dy.astype(np.float64).T @ x64) < 1e-5
    assert gpu.check_errors() == 0


@pytest.mark.parametrize("m,n,k", [(256, 1024, 784), (64, 300, 2000), (1, 37, 4096), (385, 200, 130)])
@pytest.mark.parametrize("prec,bound", [("bf16x3", 1e-5), ("bf16", 8e-3), ("fp32", 2e-6)])
def test_tile_widths_and_split_counts_agree(gpu, vk, m, n, k, prec, bound):
    """Every plan the tuner may choose (tile width 256 or 128 x split count)
    gives the precision's accuracy, the table's choice is the one used, and a
    fixed choice is bit-reproducible.  In split mode all plans give the same
    bits when K is not split (the per-element accumulation does not depend on
    the tile width)."""
    import ctypes as C
    from vulkpy_gb300 import _lib
    P = {"bf16x3": _lib.MM_BF16X3, "bf16": _lib.MM_BF16, "fp32": _lib.MM_FP32}[prec]
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((m, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    a, b = vk.Array(gpu, data=A), vk.Array(gpu, data=B)
    exp = A.astype(np.float64) @ B.T.astype(np.float64)
    unsplit = []
    try:
        for tile in (256, 128):
            for s in (1, 2, 3, 8, 16):
                assert _lib.lib.vkc_gemm_plan_set(P, m, n, k, s, tile) == 0
                got, got_tile = C.c_int(), C.c_int()
                assert _lib.lib.vkc_gemm_plan_get(gpu.handle, P, m, n, k, C.byref(got), C.byref(got_tile)) == 0
                kstep = 16 if prec == "fp32" else 64   # SIMT K step / tensor-core K block
                assert got.value == min(s, (k + kstep - 1) // kstep)
                assert got_tile.value == (128 if prec == "fp32" else tile)   # the SIMT GEMM has one tile
                outs = []
                for _ in range(2):
                    c = vk.Array(gpu, shape=(m, n))
                    st = _lib.lib.vkc_gemm(gpu.handle, P, 0, 1, m, n, k, C.c_float(1.0), a._dptr(), k,
                                           b._dptr(), k, C.c_float(0.0), c._dptr(), n)
                    assert st == 0, _lib.last_error()
                    c._written()
                    outs.append(np.asarray(c).copy())
                assert np.array_equal(outs[0], outs[1]), (tile, s)
                assert rel_fro(outs[0], exp) < bound, (tile, s)
                if s == 1:
                    unsplit.append(outs[0])
        np.testing.assert_array_equal(unsplit[0], unsplit[1])   # fp32: the same kernel twice
    finally:
        _lib.lib.vkc_gemm_tune_set(P, m, n, k, 0)
        from vulkpy_gb300 import autotune
        autotune.load_table()
    assert gpu.check_errors() == 0


@pytest.mark.parametrize("m,n,k", [(256, 1024, 784), (256, 10, 1024), (129, 300, 700), (40, 520, 1100)])
@pytest.mark.parametrize("prec", ["bf16x3", "bf16"])
def test_cluster_splitk_matches_reduction_launch(gpu, vk, m, n, k, prec):
    """Split-K reduced inside the GEMM by the CTAs of a cluster gives the bits
    of the separate reduction launch (same sums in K-range order, same
    epilogue), for 2..8 K ranges, tile widths 128 and 256, with bias,
    activation and beta."""
    import ctypes as C
    from vulkpy_gb300 import _lib, autotune
    P = {"bf16x3": _lib.MM_BF16X3, "bf16": _lib.MM_BF16}[prec]
    rng = np.random.default_rng(m * 3 + n + k)
    A = rng.standard_normal((m, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    C0 = rng.standard_normal((m, n)).astype(np.float32)
    bias = rng.standard_normal(n).astype(np.float32)
    a, b, bb = vk.Array(gpu, data=A), vk.Array(gpu, data=B), vk.Array(gpu, data=bias)
    exp = A.astype(np.float64) @ B.T.astype(np.float64)

    def run(alpha, beta, with_bias, act):
        c = vk.Array(gpu, data=C0)
        if with_bias or act:
            st = _lib.lib.vkc_dense_forward(gpu.handle, P, a._dptr(), b._dptr(), bb._dptr() if with_bias else None,
                                            c._dptr(), m, k, n, act)
        else:
            st = _lib.lib.vkc_gemm(gpu.handle, P, 0, 1, m, n, k, C.c_float(alpha), a._dptr(), k, b._dptr(), k,
                                   C.c_float(beta), c._dptr(), n)
        assert st == 0, _lib.last_error()
        c._written()
        return np.asarray(c).copy()

    try:
        for tile in (128, 256):
            for s in (2, 3, 5, 8):
                assert _lib.lib.vkc_gemm_plan_set(P, m, n, k, s, tile) == 0
                for args in ((1.0, 0.0, False, 0), (0.5, 2.0, False, 0), (1.0, 0.0, True, _lib.ACT_RELU),
                             (1.0, 0.0, True, _lib.ACT_SIGMOID)):
                    _lib.lib.vkc_set_cluster_splitk(1)
                    got = run(*args)
                    _lib.lib.vkc_set_cluster_splitk(0)
                    ref = run(*args)
                    np.testing.assert_array_equal(got, ref, err_msg=str((tile, s, args)))
                    if args == (1.0, 0.0, False, 0):
                        assert rel_fro(got, exp) < (1e-5 if prec == "bf16x3" else 8e-3)
    finally:
        _lib.lib.vkc_set_cluster_splitk(0)   # the default
        _lib.lib.vkc_gemm_tune_set(P, m, n, k, 0)
        autotune.load_table()
    assert gpu.check_errors() == 0
