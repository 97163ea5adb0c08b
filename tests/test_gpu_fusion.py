"""Fused elementwise kernels are bit-identical to running the ops one by one
(same float32 roundings: the generated code is compiled without FMA
contraction and calls the same math functions)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


@pytest.mark.parametrize("n", [1, 5, 4096, 100003])
def test_chain32_fused_equals_per_op(gpu, vk, n):
    import bench
    rng = np.random.default_rng(n)
    x = vk.Array(gpu, data=rng.standard_normal(n).astype(np.float32))
    y = vk.Array(gpu, data=rng.uniform(0.5, 2.0, n).astype(np.float32))
    f = vk.fusion.fuse(bench.chain32)
    np.testing.assert_array_equal(np.asarray(f(x, y)), np.asarray(bench.chain32(x, y)))


def test_multi_output_scalars_and_repeated_inputs(gpu, vk):
    rng = np.random.default_rng(1)
    a = vk.Array(gpu, data=rng.uniform(0.1, 3.0, (33, 65)).astype(np.float32))
    b = vk.Array(gpu, data=rng.standard_normal((33, 65)).astype(np.float32))

    def g(p, q):
        s = (p * q + 1.0) / (2.0 - q.abs())
        return s, p ** 2.0, 1.5 ** q, (p + p).invsqrt(), s.clamp(-1.0, 1.0)

    def g4(p, q):
        r = g(p, q)
        return r[0], r[1], r[2], r[3]

    f = vk.fusion.fuse(g4)
    got = f(a, b)
    exp = g4(a, b)
    for u, v in zip(got, exp):
        np.testing.assert_array_equal(np.asarray(u), np.asarray(v))
    # same array passed twice
    h = vk.fusion.fuse(lambda p, q: p * q - q)
    np.testing.assert_array_equal(np.asarray(h(a, a)), np.asarray(a * a - a))


def test_fused_kernel_inside_a_graph(gpu, vk):
    x = vk.Array(gpu, data=np.linspace(-1, 1, 1000, dtype=np.float32))
    f = vk.fusion.fuse(lambda p: (p * 3.0).tanh() + p)
    f(x)  # compile before capturing
    g = vk.graph.Graph(gpu)
    with g:
        y = f(x)
    g.launch()
    np.testing.assert_array_equal(np.asarray(y), np.asarray((x * 3.0).tanh() + x))
