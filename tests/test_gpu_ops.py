"""Parity of the CUDA kernels with the oracle on seeded inputs, at sizes the
oracle finishes in seconds, plus edge cases (ragged tails, unit and empty
dims, many broadcast patterns, out-of-range indices).

Tolerances:
  * + - * / max min, broadcast copies, clamp, gather, PRNG integers: bit-exact.
  * unary math: within the CUDA math library's documented ulp bound of the
    float64 result (ULP_BOUND below, +1 for rounding of the reference value).
  * sums: |err| <= 2^-22 * sum|x| (compensated summation); prod: rel 1e-5.
  * fp32 matmul: relative Frobenius error vs float64 <= 1e-6.
"""
import zlib

import numpy as np
import pytest

from oracle import ops as O

pytestmark = pytest.mark.gpu

ULP_BOUND = {"abs": 0, "sign": 0, "sin": 2, "cos": 2, "tan": 4, "asin": 2, "acos": 2, "atan": 2, "sinh": 3,
             "cosh": 2, "tanh": 2, "asinh": 3, "acosh": 4, "atanh": 3, "exp": 2, "log": 1, "exp2": 2,
             "log2": 1, "sqrt": 0, "invsqrt": 1}
DOMAIN = {"asin": (-1, 1), "acos": (-1, 1), "atanh": (-0.99, 0.99), "acosh": (1, 50), "log": (1e-3, 100),
          "log2": (1e-3, 100), "sqrt": (0, 100), "invsqrt": (1e-3, 100), "exp": (-80, 80), "exp2": (-100, 100),
          "sinh": (-80, 80), "cosh": (-80, 80), "tan": (-1.5, 1.5)}
TRUTH = {"abs": np.abs, "sign": np.sign, "sin": np.sin, "cos": np.cos, "tan": np.tan, "asin": np.arcsin,
         "acos": np.arccos, "atan": np.arctan, "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh,
         "asinh": np.arcsinh, "acosh": np.arccosh, "atanh": np.arctanh, "exp": np.exp, "log": np.log,
         "exp2": np.exp2, "log2": np.log2, "sqrt": np.sqrt, "invsqrt": lambda x: 1 / np.sqrt(x)}

BIN = {"add": (O.ADD, "__add__"), "sub": (O.SUB, "__sub__"), "mul": (O.MUL, "__mul__"),
       "div": (O.DIV, "__truediv__"), "max": (O.MAX, "max"), "min": (O.MIN, "min")}


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


@pytest.mark.parametrize("n", [1, 3, 4, 7, 1000, 100003])
@pytest.mark.parametrize("name", list(BIN))
def test_binary_same_shape(gpu, vk, name, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n).astype(np.float32)
    b = rng.standard_normal(n).astype(np.float32) + 0.1
    op, meth = BIN[name]
    x, y = vk.Array(gpu, data=a), vk.Array(gpu, data=b)
    np.testing.assert_array_equal(np.asarray(getattr(x, meth)(y)), O.binary(op, a, b))
    # in place
    if name in ("add", "sub", "mul", "div"):
        getattr(x, "__i" + meth[2:])(y)
    else:
        getattr(x, meth)(y, inplace=True)
    np.testing.assert_array_equal(np.asarray(x), O.binary(op, a, b))


@pytest.mark.parametrize("s", [2.0, -0.75, 3.0])
def test_scalar_and_reversed(gpu, vk, s):
    rng = np.random.default_rng(1)
    a = rng.uniform(0.1, 2.0, 10001).astype(np.float32)
    x = vk.Array(gpu, data=a)
    np.testing.assert_array_equal(np.asarray(x + s), O.scalar(O.ADD, a, s))
    np.testing.assert_array_equal(np.asarray(x - s), O.scalar(O.SUB, a, s))
    np.testing.assert_array_equal(np.asarray(x * s), O.scalar(O.MUL, a, s))
    np.testing.assert_array_equal(np.asarray(x / s), O.scalar(O.DIV, a, s))
    np.testing.assert_array_equal(np.asarray(s - x), O.scalar(O.RSUB, a, s))
    np.testing.assert_array_equal(np.asarray(s / x), O.scalar(O.RDIV, a, s))
    np.testing.assert_array_equal(np.asarray(x.max(s)), O.scalar(O.MAX, a, s))
    np.testing.assert_array_equal(np.asarray(x.min(s)), O.scalar(O.MIN, a, s))
    p = np.asarray(x ** s)
    assert O.ulp_distance(p, a.astype(np.float64) ** s).max() <= 3
    q = np.asarray(abs(s) ** x)
    assert O.ulp_distance(q, abs(s) ** a.astype(np.float64)).max() <= 3


def test_pow_arrays(gpu, vk):
    rng = np.random.default_rng(2)
    a = rng.uniform(0.1, 3, 5000).astype(np.float32)
    b = rng.uniform(-3, 3, 5000).astype(np.float32)
    got = np.asarray(vk.Array(gpu, data=a) ** vk.Array(gpu, data=b))
    assert O.ulp_distance(got, a.astype(np.float64) ** b.astype(np.float64)).max() <= 3


@pytest.mark.parametrize("name", list(ULP_BOUND))
def test_unary_math_ulp(gpu, vk, name):
    rng = np.random.default_rng(7)
    lo, hi = DOMAIN.get(name, (-10, 10))
    a = rng.uniform(lo, hi, 65537).astype(np.float32)
    x = vk.Array(gpu, data=a)
    got = np.asarray(getattr(x, name)())
    truth = TRUTH[name](a.astype(np.float64))
    d = O.ulp_distance(got, truth)
    assert d.max() <= ULP_BOUND[name] + 1, (name, d.max())
    getattr(x, name)(inplace=True)
    np.testing.assert_array_equal(np.asarray(x), got)


def _random_shapes(rng, count):
    pairs = []
    for _ in range(count):
        nd = int(rng.integers(1, 6))
        out = rng.integers(1, 6, nd)
        if rng.random() < 0.3:
            out[-1] = int(rng.integers(64, 300))
        a = [d if rng.random() < 0.6 else 1 for d in out]
        b = [d if rng.random() < 0.6 else 1 for d in out]
        a = a[int(rng.integers(0, nd)):] if rng.random() < 0.3 else a
        b = b[int(rng.integers(0, nd)):] if rng.random() < 0.3 else b
        pairs.append((tuple(a) or (1,), tuple(b) or (1,)))
    return pairs


@pytest.mark.parametrize("case", range(40))
def test_broadcast_binary_random_shapes(gpu, vk, case):
    rng = np.random.default_rng(100 + case)
    sa, sb = _random_shapes(rng, 1)[0]
    a = rng.standard_normal(sa).astype(np.float32)
    b = rng.standard_normal(sb).astype(np.float32) + 0.05
    x, y = vk.Array(gpu, data=a), vk.Array(gpu, data=b)
    for name, (op, meth) in BIN.items():
        got = np.asarray(getattr(x, meth)(y))
        np.testing.assert_array_equal(got, O.bcast(op, a, b), err_msg=f"{name} {sa} {sb}")
    shape = np.broadcast_shapes(sa, sb)
    if shape == tuple(a.shape):
        z = vk.Array(gpu, data=a)
        z += y
        np.testing.assert_array_equal(np.asarray(z), O.bcast(O.ADD, a, b))
    t = np.asarray(x.broadcast_to(shape))
    np.testing.assert_array_equal(t, np.broadcast_to(a, shape))


def test_broadcast_large_row_and_col(gpu, vk):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((257, 4100)).astype(np.float32)
    row = rng.uniform(0.5, 2, (1, 4100)).astype(np.float32)
    col = rng.uniform(0.5, 2, (257, 1)).astype(np.float32)
    x = vk.Array(gpu, data=X)
    for other in (row, col):
        o = vk.Array(gpu, data=other)
        for name, (op, meth) in BIN.items():
            np.testing.assert_array_equal(np.asarray(getattr(x, meth)(o)), O.bcast(op, X, other))
        got = np.asarray(x ** o)
        with np.errstate(invalid="ignore"):
            truth = X.astype(np.float64) ** other.astype(np.float64)
        fin = np.isfinite(truth)
        assert np.array_equal(np.isfinite(got), fin)
        assert O.ulp_distance(got[fin], truth[fin]).max() <= 3
        # in place: the output is the first operand (full 4096-column chunks
        # and the 4-column tail)
        for op, meth in ((O.DIV, "__itruediv__"), (O.ADD, "__iadd__")):
            z = vk.Array(gpu, data=X)
            getattr(z, meth)(o)
            np.testing.assert_array_equal(np.asarray(z), O.bcast(op, X, other))
        z = vk.Array(gpu, data=np.abs(X) + 0.5)
        z **= o
        np.testing.assert_array_equal(np.asarray(z), np.asarray(vk.Array(gpu, data=np.abs(X) + 0.5) ** o))


@pytest.mark.parametrize("shape,other", [((37, 8192), (1, 8192)), ((37, 8192), (37, 1)), ((3, 5, 4096), (5, 1)),
                                         ((2, 3, 12288), (1, 3, 12288)), ((1, 4096), (1, 1))])
def test_inplace_broadcast_full_chunks(gpu, vk, shape, other):
    """In place with whole 4096-column chunks (the kernel that loads a
    block's next chunk before storing the current one): bit-exact with the
    oracle for + - * / max min, ** equal to the out-of-place result, and an
    in-place clamp with broadcast bounds."""
    rng = np.random.default_rng(sum(shape))
    X = rng.standard_normal(shape).astype(np.float32)
    Y = rng.uniform(0.5, 2, other).astype(np.float32)
    y = vk.Array(gpu, data=Y)
    for op, meth in ((O.ADD, "__iadd__"), (O.SUB, "__isub__"), (O.MUL, "__imul__"), (O.DIV, "__itruediv__")):
        z = vk.Array(gpu, data=X)
        getattr(z, meth)(y)
        np.testing.assert_array_equal(np.asarray(z), O.bcast(op, X, Y))
    for op, meth in ((O.MAX, "max"), (O.MIN, "min")):
        z = vk.Array(gpu, data=X)
        getattr(z, meth)(y, inplace=True)
        np.testing.assert_array_equal(np.asarray(z), O.bcast(op, X, Y))
    z = vk.Array(gpu, data=np.abs(X) + 0.5)
    z **= y
    np.testing.assert_array_equal(np.asarray(z), np.asarray(vk.Array(gpu, data=np.abs(X) + 0.5) ** y))
    lo = vk.Array(gpu, data=-Y)
    hi = vk.Array(gpu, data=Y * 0.5)
    z = vk.Array(gpu, data=X)
    z.clamp(lo, hi, inplace=True)
    np.testing.assert_array_equal(np.asarray(z), np.minimum(np.maximum(X, -Y), Y * 0.5))
    assert gpu.check_errors() == 0


def test_clamp_variants(gpu, vk):
    rng = np.random.default_rng(8)
    a = rng.standard_normal((33, 70)).astype(np.float32)
    lo = rng.uniform(-1, 0, (33, 70)).astype(np.float32)
    hi = rng.uniform(0, 1, (1, 70)).astype(np.float32)
    x = vk.Array(gpu, data=a)
    np.testing.assert_array_equal(np.asarray(x.clamp(-0.5, 0.5)), O.clamp(a, -0.5, 0.5))
    np.testing.assert_array_equal(np.asarray(x.clamp(vk.Array(gpu, data=lo), 0.5)), O.clamp(a, lo, 0.5))
    np.testing.assert_array_equal(np.asarray(x.clamp(-0.5, vk.Array(gpu, data=hi))), O.clamp(a, -0.5, hi))
    np.testing.assert_array_equal(np.asarray(x.clamp(vk.Array(gpu, data=lo), vk.Array(gpu, data=hi))),
                                  O.clamp(a, lo, hi))
    x.clamp(vk.Array(gpu, data=lo), vk.Array(gpu, data=hi), inplace=True)
    np.testing.assert_array_equal(np.asarray(x), O.clamp(a, lo, hi))


SHAPES_AXES = [((7,), 0), ((513, 129), 0), ((513, 129), 1), ((3, 4100), 1), ((4100, 3), 0), ((2, 3, 4, 5), (1, 2)),
               ((2, 3, 4, 2, 2, 4, 3), (1, 2, 5)), ((64, 64, 64), (0, 2)), ((5, 70001), 1), ((70001, 2), 0),
               ((1, 300000), 1), ((300000, 1), 0), ((9, 17), -1), ((512, 1024), 0), ((3, 700, 36), 1),
               ((2100, 6), 0)]


@pytest.mark.parametrize("shape,axis", SHAPES_AXES)
@pytest.mark.parametrize("red", ["sum", "prod", "maximum", "minimum", "mean"])
def test_axis_reductions(gpu, vk, shape, axis, red):
    rng = np.random.default_rng(zlib.crc32(repr((shape, axis)).encode()))
    if red == "prod":
        a = rng.uniform(0.9995, 1.0005, shape).astype(np.float32)
    else:
        a = rng.standard_normal(shape).astype(np.float32)
    x = vk.Array(gpu, data=a)
    got = np.asarray(getattr(x, red)(axis=axis))
    a64 = a.astype(np.float64)
    ax = axis if isinstance(axis, tuple) else (axis,)
    if red in ("maximum", "minimum"):
        exp = a.max(axis=ax) if red == "maximum" else a.min(axis=ax)
        np.testing.assert_array_equal(got, exp)
    elif red == "prod":
        np.testing.assert_allclose(got, a64.prod(axis=ax), rtol=1e-5)
    else:
        exp = a64.sum(axis=ax)
        bound = np.abs(a64).sum(axis=ax) * 2.0 ** -21 + 1e-30
        if red == "mean":
            n = a.size // max(1, exp.size)
            exp = exp / n
            bound = bound / n * 2
        assert np.all(np.abs(got - exp) <= bound), np.max(np.abs(got - exp) / bound)
    keep = np.asarray(getattr(x, red)(axis=axis, keepdims=True))
    assert keep.shape == np.sum(a, axis=ax, keepdims=True).shape


@pytest.mark.parametrize("n", [1, 5, 4096, 4097, 1 << 20, (1 << 24) + 3])
def test_full_reductions(gpu, vk, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n).astype(np.float32)
    x = vk.Array(gpu, data=a)
    s = float(np.asarray(x.sum())[0])
    assert abs(s - np.sum(a, dtype=np.float64)) <= np.abs(a).sum(dtype=np.float64) * 2.0 ** -23 + 1e-6
    np.testing.assert_allclose(np.asarray(x.mean()), [np.mean(a, dtype=np.float64)], rtol=1e-5, atol=1e-7)
    assert np.asarray(x.maximum())[0] == a.max()
    assert np.asarray(x.minimum())[0] == a.min()
    p = rng.uniform(0.99999, 1.00001, n).astype(np.float32)
    got = np.asarray(vk.Array(gpu, data=p).prod())[0]
    np.testing.assert_allclose(got, np.prod(p, dtype=np.float64), rtol=2e-5)


@pytest.mark.parametrize("shape", [(37, 300), (600, 64), (700, 30)])
def test_rebroadcast(gpu, vk, shape):
    rng = np.random.default_rng(3)
    a = rng.standard_normal(shape).astype(np.float32)
    x = vk.Array(gpu, data=a)
    for axis in (0, 1):
        got = np.asarray(x.maximum(axis=axis, rebroadcast=True))
        np.testing.assert_array_equal(got, np.broadcast_to(a.max(axis=axis, keepdims=True), a.shape))
        s = np.asarray(x.sum(axis=axis, rebroadcast=True))
        np.testing.assert_allclose(s, np.broadcast_to(a.astype(np.float64).sum(axis=axis, keepdims=True), a.shape),
                                   rtol=1e-5, atol=1e-5)
        m = np.asarray(x.mean(axis=axis, rebroadcast=True))
        np.testing.assert_allclose(m, np.broadcast_to(a.astype(np.float64).mean(axis=axis, keepdims=True), a.shape),
                                   rtol=1e-5, atol=1e-6)


def test_gather_flat_and_axis(gpu, vk):
    rng = np.random.default_rng(11)
    a = rng.standard_normal((64, 33, 10)).astype(np.float32)
    idx = rng.integers(0, a.size, 10007).astype(np.uint32)
    x = vk.Array(gpu, data=a)
    np.testing.assert_array_equal(np.asarray(x.gather(vk.U32Array(gpu, data=idx))), O.gather(a, idx))
    for axis in (0, 1, 2):
        ii = rng.integers(0, a.shape[axis], (5, 3)).astype(np.uint32)
        got = np.asarray(x.gather(vk.U32Array(gpu, data=ii), axis=axis))
        np.testing.assert_array_equal(got, O.gather_axis(a, ii, axis))
        # numpy take, with the index axes moved to the front
        exp = np.moveaxis(np.take(a, ii.astype(np.int64), axis=axis), list(range(axis, axis + 2)), [0, 1])
        np.testing.assert_array_equal(got, exp)
    big = vk.Array(gpu, data=rng.standard_normal((300, 1000)).astype(np.float32))
    ii = rng.integers(0, 300, 77).astype(np.uint32)
    np.testing.assert_array_equal(np.asarray(big.gather(vk.U32Array(gpu, data=ii), axis=0)),
                                  np.asarray(big)[ii.astype(np.int64)])


def test_gather_out_of_range_sets_flag(gpu, vk):
    gpu.check_errors()  # clear
    a = vk.Array(gpu, data=np.arange(10, dtype=np.float32))
    out = np.asarray(a.gather(vk.U32Array(gpu, data=[1, 10, 3, 4000000000])))
    assert out[0] == 1 and out[2] == 3 and np.isnan(out[1]) and np.isnan(out[3])
    assert gpu.check_errors() & 1
    assert gpu.check_errors() == 0


@pytest.mark.parametrize("size", [1, 2, 3, 64, 1000, 4096])
@pytest.mark.parametrize("n", [1, 63, 64, 65, 4097, 100000])
def test_prng_bit_exact(gpu, vk, size, n):
    r = vk.random.Xoshiro128pp(gpu, size=size, seed=size * 7919 + n)
    ref = O.Xoshiro128pp(size * 7919 + n, size)
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)
    np.testing.assert_array_equal(np.asarray(r.randint(shape=(n,))), ref.u32(n))
    np.testing.assert_array_equal(np.asarray(r.random(shape=(n,))), ref.f32(n))
    np.testing.assert_array_equal(np.asarray(r.randrange(shape=(n,), low=3, high=1000)), ref.randrange(n, 3, 1000))
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)


@pytest.mark.parametrize("size", [2, 3, 64, 1001])
@pytest.mark.parametrize("n", [1, 2, 11, 128, 129, 50000])
def test_prng_normal(gpu, vk, size, n):
    r = vk.random.Xoshiro128pp(gpu, size=size, seed=5)
    ref = O.Xoshiro128pp(5, size)
    got = np.asarray(r.normal(shape=(n,), mean=1.5, stddev=2.0))
    exp = ref.normal(n, 1.5, 2.0)
    # same uniforms; Box-Muller through CUDA vs glibc logf/sinf/cosf
    np.testing.assert_allclose(got, exp, rtol=2e-6, atol=4e-6)
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)


def test_prng_large_seed_state(gpu, vk):
    r = vk.random.Xoshiro128pp(gpu, size=70000, seed=1)
    ref = O.Xoshiro128pp(1, 70000)
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)


@pytest.mark.parametrize("m,k,n", [(1, 1, 1), (2, 2, 2), (17, 33, 65), (128, 128, 128), (129, 257, 131),
                                   (256, 256, 256), (300, 1, 200), (1, 700, 1), (1000, 64, 3)])
def test_matmul_fp32(gpu, vk, m, k, n):
    rng = np.random.default_rng(m * 1000 + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((k, n)).astype(np.float32)
    got = np.asarray(vk.Array(gpu, data=a) @ vk.Array(gpu, data=b))
    assert O.rel_fro(got, a.astype(np.float64) @ b.astype(np.float64)) < 1e-6


def test_matmul_vector_forms(gpu, vk):
    rng = np.random.default_rng(4)
    A = rng.standard_normal((50, 40)).astype(np.float32)
    v = rng.standard_normal(40).astype(np.float32)
    w = rng.standard_normal(50).astype(np.float32)
    np.testing.assert_allclose(np.asarray(vk.Array(gpu, data=A) @ vk.Array(gpu, data=v)), A @ v, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(np.asarray(vk.Array(gpu, data=w) @ vk.Array(gpu, data=A)), w @ A, rtol=1e-5, atol=1e-5)
    with pytest.raises(ValueError):
        vk.Array(gpu, data=A) @ vk.Array(gpu, data=A)


@pytest.mark.parametrize("size,n", [(1, 20000), (2, 300000), (64, 65536), (64, 65537), (6, 1 << 20), (1000, 777777),
                                    (64, 1 << 20)])
def test_prng_segmented_streams(gpu, vk, size, n):
    """Few states, long streams: generation is split into segments whose
    start states come from powers of the next() map; the outputs and the
    final states are those of the serial chain (bit-exact with the oracle),
    and a second call continues the stream."""
    r = vk.random.Xoshiro128pp(gpu, size=size, seed=11)
    ref = O.Xoshiro128pp(11, size)
    np.testing.assert_array_equal(np.asarray(r.randint(shape=(n,))), ref.u32(n))
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)
    np.testing.assert_array_equal(np.asarray(r.random(shape=(n // 3,))), ref.f32(n // 3))
    np.testing.assert_array_equal(r.state().reshape(-1), ref.state)
    if size % 2 == 0:
        got = np.asarray(r.normal(shape=(n // 2,), mean=0.5, stddev=3.0))
        np.testing.assert_allclose(got, ref.normal(n // 2, 0.5, 3.0), rtol=2e-6, atol=6e-6)
        np.testing.assert_array_equal(r.state().reshape(-1), ref.state)


def test_pow_accuracy_wide_ranges(gpu, vk):
    """pow (CUDA's powf) against float64: within its documented 4 ulp over
    wide ranges, |x| near 1 with large |y|, negative x with integer y (sign
    of odd powers), NaN for negative x with non-integer y, and the special
    values (0, inf, NaN, overflow and underflow)."""
    rng = np.random.default_rng(42)
    n = 1 << 18
    x = np.concatenate([
        rng.uniform(-2, 2, n), np.exp(rng.uniform(-40, 40, n)), 1 + rng.uniform(-5e-3, 5e-3, n),
        -rng.uniform(0.01, 10, n)]).astype(np.float32)
    y = np.concatenate([
        rng.uniform(0.5, 2, n), rng.uniform(-3, 3, n), rng.uniform(-2e4, 2e4, n),
        rng.integers(-20, 21, n).astype(np.float64)]).astype(np.float32)
    got = np.asarray(vk.Array(gpu, data=x) ** vk.Array(gpu, data=y))
    with np.errstate(all="ignore"):
        truth = np.power(x.astype(np.float64), y.astype(np.float64))
    nan = np.isnan(truth)
    np.testing.assert_array_equal(np.isnan(got), nan)
    fin = ~nan & (np.abs(truth) < 3.4e38) & (np.abs(truth) > 1.2e-38)
    assert O.ulp_distance(got[fin], truth[fin]).max() <= 4.0
    over = ~nan & (np.abs(truth) >= 3.5e38)
    assert np.all(np.isinf(got[over]) & (np.sign(got[over]) == np.sign(truth[over])))
    sx = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 2.0, 2.0, 2.0, 0.5, 1.0], np.float32)
    sy = np.array([2.0, 3.0, 0.5, 3.0, 1.0, np.inf, -np.inf, 0.0, 200.0, np.nan], np.float32)
    gs = np.asarray(vk.Array(gpu, data=sx) ** vk.Array(gpu, data=sy))
    with np.errstate(all="ignore"):
        es = np.power(sx, sy)
    np.testing.assert_array_equal(gs, es)
