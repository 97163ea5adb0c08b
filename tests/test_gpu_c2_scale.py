"""Parity at the bandwidth suite's own sizes (X: 8192 x 32768 float32 N(0,1),
row (1, 32768) and col (8192, 1) uniform[0.5, 2), 2^26 gather indices,
Xoshiro128pp with 2^20 states producing 2^28 outputs), the inputs that
bench.py times, drawn the same way (numpy default_rng(0), in that order).

Code paths that only large inputs reach are checked here: the 4096-column
broadcast chunks of 32768-wide rows, the column-split axis reductions, the
float64 cross-block combine of full reductions over 2^28 elements, the
many-state generator (four draws per thread) and the fused Box-Muller pass
over 2^19-pair launches.

Tolerances (the same as the small-size tests):
  * + - * / max min (out of place and in place), gather, the raw u32 and
    float streams and the generator states: bit-exact with the oracle.
  * pow: NaN pattern equal, finite results within 3 ulp of float64.
  * sqrt within 0.5 ulp of float64 (correctly rounded), invsqrt 2, log 2
    ulp (CUDA's documented bounds + 1).
  * sum / mean: |err| <= 2^-21 sum|x| (axis) or 2^-23 sum|x| (axis=None),
    maximum / minimum exact, prod rel 2e-5 of float64.
  * normals: rtol 2e-6, atol 4e-6 (CUDA vs glibc logf/sinf/cosf on the same
    uniforms).
"""
import gc

import numpy as np
import pytest

from oracle import ops as O

pytestmark = pytest.mark.gpu

ROWS, COLS = 8192, 32768
N_IDX = 1 << 26
STATES = 1 << 20
N_OUT = ROWS * COLS

BIN = [("__add__", O.ADD), ("__sub__", O.SUB), ("__mul__", O.MUL), ("__truediv__", O.DIV), ("max", O.MAX),
       ("min", O.MIN)]


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


@pytest.fixture(scope="module")
def host_inputs():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((ROWS, COLS), dtype=np.float32)
    row = rng.uniform(0.5, 2.0, (1, COLS)).astype(np.float32)
    col = rng.uniform(0.5, 2.0, (ROWS, 1)).astype(np.float32)
    idx = rng.integers(0, ROWS * COLS, N_IDX, dtype=np.uint32)
    return X, row, col, idx


@pytest.fixture(scope="module")
def dev_inputs(gpu, vk, host_inputs):
    X, row, col, idx = host_inputs
    d = (vk.Array(gpu, data=X), vk.Array(gpu, data=row), vk.Array(gpu, data=col), vk.U32Array(gpu, data=idx))
    yield d
    del d
    gc.collect()
    gpu.wait()


@pytest.mark.parametrize("which", ["row", "col"])
def test_broadcast_binary_full_size(gpu, vk, host_inputs, dev_inputs, which):
    X, row, col, _ = host_inputs
    x, r, c, _ = dev_inputs
    other, o = (row, r) if which == "row" else (col, c)
    for meth, op in BIN:
        got = np.asarray(getattr(x, meth)(o))
        exp = O.bcast(op, X, other)
        assert np.array_equal(got, exp), (meth, which, int(np.count_nonzero(got != exp)))
        del got, exp
    got = np.asarray(x ** o)
    with np.errstate(invalid="ignore"):
        truth = np.power(X.astype(np.float64), other.astype(np.float64))
    fin = np.isfinite(truth)
    assert np.array_equal(np.isfinite(got), fin)
    assert O.ulp_distance(got[fin], truth[fin]).max() <= 3
    del got, truth, fin


def test_unary_full_size(gpu, vk, host_inputs, dev_inputs):
    X = host_inputs[0]
    x = dev_inputs[0]
    z = x.abs()
    z += 1e-3
    Z = np.abs(X) + np.float32(1e-3)
    np.testing.assert_array_equal(np.asarray(z), Z)
    Z64 = Z.astype(np.float64)
    for name, truth, bound in (("sqrt", np.sqrt, 0.5), ("invsqrt", lambda t: 1.0 / np.sqrt(t), 2),
                               ("log", np.log, 2)):
        got = np.asarray(getattr(z, name)())
        d = O.ulp_distance(got, truth(Z64))
        assert d.max() <= bound, (name, float(d.max()))
        del got, d
    s = np.asarray(z.sqrt())
    z.sqrt(inplace=True)
    np.testing.assert_array_equal(np.asarray(z), s)


@pytest.mark.parametrize("axis", [0, 1, None])
def test_reductions_full_size(gpu, vk, host_inputs, dev_inputs, axis):
    X = host_inputs[0]
    x = dev_inputs[0]
    X64 = X.astype(np.float64)
    exp_sum = X64.sum(axis=axis)
    abs_sum = np.abs(X64).sum(axis=axis)
    k = 2.0 ** -23 if axis is None else 2.0 ** -21
    got = np.asarray(x.sum(axis=axis)).astype(np.float64).reshape(np.shape(exp_sum))
    assert np.all(np.abs(got - exp_sum) <= abs_sum * k + 1e-30)
    n = X.size // max(1, np.size(exp_sum))
    got = np.asarray(x.mean(axis=axis)).astype(np.float64).reshape(np.shape(exp_sum))
    assert np.all(np.abs(got - exp_sum / n) <= abs_sum / n * 2 * k + 1e-30)
    np.testing.assert_array_equal(np.asarray(x.maximum(axis=axis)).reshape(np.shape(exp_sum)), X.max(axis=axis))
    np.testing.assert_array_equal(np.asarray(x.minimum(axis=axis)).reshape(np.shape(exp_sum)), X.min(axis=axis))
    del X64
    # prod of E = exp(X * 1e-4): E itself exact through the scalar and
    # in-place exp kernels is checked by the element-wise tests; here the
    # device E is compared with float64 truth of its product
    e = x * 1e-4
    e.exp(inplace=True)
    E = np.asarray(e).astype(np.float64)
    got = np.asarray(e.prod(axis=axis)).astype(np.float64).reshape(np.shape(exp_sum))
    np.testing.assert_allclose(got, E.prod(axis=axis), rtol=2e-5)


def test_gather_full_size(gpu, vk, host_inputs, dev_inputs):
    X, _, _, idx = host_inputs
    x, _, _, i = dev_inputs
    gpu.check_errors()
    got = np.asarray(x.gather(i))
    np.testing.assert_array_equal(got, X.reshape(-1)[idx.astype(np.int64)])
    assert gpu.check_errors() == 0


def test_prng_full_size(gpu, vk):
    """2^20 states, seed 0: 2^28 floats, 2^28 normals and 2^28 raw u32 in the
    order the benchmark draws them; states after each call."""
    r = vk.random.Xoshiro128pp(gpu, size=STATES, seed=0)
    ref = O.Xoshiro128pp(0, STATES)
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)
    U = vk.Array(gpu, shape=(N_OUT,))
    r.random(buffer=U)
    np.testing.assert_array_equal(np.asarray(U), ref.f32(N_OUT))
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)
    r.normal(buffer=U)
    np.testing.assert_allclose(np.asarray(U), ref.normal(N_OUT), rtol=2e-6, atol=4e-6)
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)
    del U
    I = vk.U32Array(gpu, shape=(N_OUT,))
    r.randint(buffer=I)
    np.testing.assert_array_equal(np.asarray(I), ref.u32(N_OUT))
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)


def test_inplace_broadcast_full_size(gpu, vk, host_inputs):
    """The eight in-place broadcasts of the suite in its order, applied to
    one array: X op= row for + - * /, then X op= col."""
    X, row, col, _ = host_inputs
    x = vk.Array(gpu, data=X)
    r, c = vk.Array(gpu, data=row), vk.Array(gpu, data=col)
    exp = X.copy()
    for other, o in ((row, r), (col, c)):
        for meth, op in (("__iadd__", O.ADD), ("__isub__", O.SUB), ("__imul__", O.MUL), ("__itruediv__", O.DIV)):
            getattr(x, meth)(o)
            exp = O.bcast(op, exp, other)
            got = np.asarray(x)
            assert np.array_equal(got, exp), (meth, int(np.count_nonzero(got != exp)))
            del got
