"""argmax / argmin and the device permutation / shuffle.

argmax/argmin: numpy is the specification (first index of the extreme value,
the first NaN if there is one, -0.0 == +0.0), so numpy.argmax is the oracle
and the results must match exactly.  The permutation must equal the C
restatement in oracle/vkoracle.c bit for bit and advance the generator like a
4-value draw."""
import numpy as np
import pytest

from oracle.ops import Xoshiro128pp as OracleXo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


def _data(rng, shape, ties=False, nans=0, zeros=False):
    if ties:
        a = rng.integers(-3, 4, size=shape).astype(np.float32)
    else:
        a = rng.standard_normal(shape).astype(np.float32)
    flat = a.reshape(-1)
    if zeros:
        flat[rng.integers(0, flat.size, size=max(1, flat.size // 8))] = -0.0
        flat[rng.integers(0, flat.size, size=max(1, flat.size // 8))] = 0.0
    if nans:
        flat[rng.integers(0, flat.size, size=nans)] = np.nan
    return a


@pytest.mark.parametrize("n", [1, 2, 7, 64, 1000, 4099, 1 << 20, (1 << 20) + 3])
@pytest.mark.parametrize("kind", ["normal", "ties", "nan", "zeros"])
def test_arg_all(gpu, vk, n, kind):
    rng = np.random.default_rng(n)
    a = _data(rng, (n,), ties=kind == "ties", nans=2 if kind == "nan" and n > 2 else 0, zeros=kind == "zeros")
    if kind == "zeros":
        a[:] = np.where(a > 0, -a, a)       # max is a zero: +0/-0 must tie
    x = vk.Array(gpu, data=a)
    got_max, got_min = x.argmax(), x.argmin()
    assert got_max.shape == (1,) and got_min.shape == (1,)
    assert int(np.asarray(got_max)[0]) == int(np.argmax(a)), kind
    assert int(np.asarray(got_min)[0]) == int(np.argmin(a)), kind


def test_arg_all_unaligned_and_keepdims(gpu, vk):
    rng = np.random.default_rng(5)
    a = rng.standard_normal((33, 65)).astype(np.float32)
    x = vk.Array(gpu, data=a)
    k = x.argmax(keepdims=True)
    assert k.shape == (1, 1) and int(np.asarray(k).reshape(-1)[0]) == int(np.argmax(a))
    x.reshape((33 * 65,))
    assert int(np.asarray(x.argmin())[0]) == int(np.argmin(a))


SHAPES_AXES = [
    ((512, 1024), 0), ((512, 1024), 1), ((512, 1024), -1),
    ((3, 5000), 1),                     # long rows: one block per row
    ((70, 33), 0), ((70, 33), 1),       # post not a multiple of 32
    ((4, 6, 37), 1), ((2, 3, 4, 2, 2, 4, 3), 3), ((2, 3, 4, 2, 2, 4, 3), 0),
    ((1, 1), 0), ((9,), 0), ((8192, 257), 0), ((257, 8192), 1),
]


@pytest.mark.parametrize("shape,axis", SHAPES_AXES)
@pytest.mark.parametrize("ties", [False, True])
def test_arg_axis(gpu, vk, shape, axis, ties):
    rng = np.random.default_rng(len(shape) * 100 + axis + 7)
    a = _data(rng, shape, ties=ties, nans=3 if a_size(shape) > 50 else 0)
    x = vk.Array(gpu, data=a)
    for keepdims in (False, True):
        gm = x.argmax(axis=axis, keepdims=keepdims)
        gn = x.argmin(axis=axis, keepdims=keepdims)
        em = np.argmax(a, axis=axis, keepdims=keepdims)
        en = np.argmin(a, axis=axis, keepdims=keepdims)
        assert gm.shape == em.shape and gn.shape == en.shape
        np.testing.assert_array_equal(np.asarray(gm), em.astype(np.uint32))
        np.testing.assert_array_equal(np.asarray(gn), en.astype(np.uint32))


def a_size(shape):
    return int(np.prod(shape))


def test_arg_errors(gpu, vk):
    x = vk.Array(gpu, shape=(0,))
    with pytest.raises(ValueError):
        x.argmax()
    y = vk.Array(gpu, data=np.zeros((2, 3), np.float32))
    with pytest.raises(ValueError):
        y.argmax(axis=2)
    with pytest.raises(ValueError):
        y.argmin(axis=(0, 1))


def test_arg_full_size(gpu, vk):
    """A 2^27-element array (512 MiB, larger than L2) with one planted
    maximum and one planted minimum."""
    n = 1 << 27
    r = vk.random.Xoshiro128pp(gpu, size=1 << 16, seed=0)
    x = r.random(shape=(n,))
    x[123456789] = 2.0
    x[98765432] = -1.0
    assert int(np.asarray(x.argmax())[0]) == 123456789
    assert int(np.asarray(x.argmin())[0]) == 98765432
    x.reshape((1 << 13, 1 << 14))
    z = x
    am = np.asarray(z.argmax(axis=1))
    h = np.asarray(z)
    np.testing.assert_array_equal(am, np.argmax(h, axis=1).astype(np.uint32))
    np.testing.assert_array_equal(np.asarray(z.argmin(axis=0)), np.argmin(h, axis=0).astype(np.uint32))


@pytest.mark.parametrize("size", [1, 3, 64, 1 << 12])
@pytest.mark.parametrize("n", [0, 1, 2, 5, 16, 1000, 65537, 1 << 22])
def test_permutation_matches_oracle(gpu, vk, size, n):
    seed = 11 * size + n
    g = vk.random.Xoshiro128pp(gpu, size=size, seed=seed)
    o = OracleXo(seed, size)
    p = np.asarray(g.permutation(n))
    e = o.permutation(n)
    np.testing.assert_array_equal(p, e)
    if n:
        assert np.array_equal(np.sort(p), np.arange(n, dtype=np.uint32))
    # the generator advanced exactly like the oracle's
    np.testing.assert_array_equal(g.state().reshape(-1), o.state)
    np.testing.assert_array_equal(np.asarray(g.randint(shape=(300,))), o.u32(300))


def test_shuffle_rows(gpu, vk):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((1000, 7)).astype(np.float32)
    x = vk.Array(gpu, data=a)
    g = vk.random.Xoshiro128pp(gpu, seed=5)
    g.shuffle(x)
    perm = OracleXo(5, 64).permutation(1000)
    np.testing.assert_array_equal(np.asarray(x), a[perm])
    # 1-D and trivial cases
    v = vk.Array(gpu, data=np.arange(10, dtype=np.float32))
    g.shuffle(v)
    assert sorted(np.asarray(v).tolist()) == list(range(10))
    one = vk.Array(gpu, data=np.ones((1, 4), np.float32))
    g.shuffle(one)
    np.testing.assert_array_equal(np.asarray(one), np.ones((1, 4), np.float32))
