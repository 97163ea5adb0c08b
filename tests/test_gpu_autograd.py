"""Hand-written backward kernels behind torch.autograd.Function:
  * against float64 central finite differences (h = 1e-6) of the same
    network computed in float64 (784 -> 32 -> 10, ReLU, softmax cross
    entropy), relative error of the sampled gradient <= 1e-6;
  * against this package's drop-in nn backward (vulkpy's semantics): equal.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _loss64(params, X, Y, eps=0.0):
    """Softmax cross entropy in float64.  The forward kernels use
    log(p + 1e-8) (nn_cross_entropy.comp:21-26) while the backward is
    softmax - y (losses.py:229-249), the exact gradient of the eps = 0 loss:
    finite differences are taken of that one."""
    W1, b1, W2, b2 = params
    h = np.maximum(X @ W1.T + b1, 0.0)
    z = h @ W2.T + b2
    z = z - z.max(1, keepdims=True)
    p = np.exp(z) / np.exp(z).sum(1, keepdims=True)
    return float((-Y * np.log(p + eps)).sum(1).mean())


@pytest.fixture(scope="module")
def problem():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((64, 784)).astype(np.float32)
    Y = np.eye(10, dtype=np.float32)[rng.integers(0, 10, 64)]
    W1 = (rng.standard_normal((32, 784)) * np.sqrt(2 / 784)).astype(np.float32)
    b1 = (rng.standard_normal(32) * 0.1).astype(np.float32)
    W2 = (rng.standard_normal((10, 32)) * np.sqrt(2 / 32)).astype(np.float32)
    b2 = (rng.standard_normal(10) * 0.1).astype(np.float32)
    return X, Y, [W1, b1, W2, b2]


def _torch_grads(problem, precision="fp32", dtype=None):
    import vulkpy_gb300.autograd as A
    dtype = dtype or torch.float32
    X, Y, params = problem
    dev = torch.device("cuda:0")
    t = [torch.tensor(p, device=dev, dtype=dtype, requires_grad=True) for p in params]
    x = torch.tensor(X, device=dev, dtype=dtype)
    y = torch.tensor(Y, device=dev, dtype=dtype)
    h = A.dense(x, t[0], t[1], act="relu", precision=precision)
    z = A.dense(h, t[2], t[3], precision=precision)
    loss = A.softmax_cross_entropy(z, y)
    loss.backward()
    torch.cuda.synchronize()
    return float(loss.detach()), [p.grad.cpu().numpy() for p in t]


def _fd_relative_error(problem, grads):
    X, Y, params = problem
    p64 = [p.astype(np.float64) for p in params]
    X64, Y64 = X.astype(np.float64), Y.astype(np.float64)
    rng = np.random.default_rng(2)
    h = 1e-6
    ours, fd = [], []
    for k, p in enumerate(p64):
        idx = rng.choice(p.size, size=min(p.size, 40), replace=False)
        for i in idx:
            plus = [q.copy() for q in p64]
            minus = [q.copy() for q in p64]
            plus[k].flat[i] += h
            minus[k].flat[i] -= h
            fd.append((_loss64(plus, X64, Y64) - _loss64(minus, X64, Y64)) / (2 * h))
            ours.append(grads[k].flat[i])
    ours, fd = np.array(ours), np.array(fd)
    return np.linalg.norm(ours - fd) / np.linalg.norm(fd)


def test_fp64_kernels_match_fp64_finite_differences(problem):
    """The hand-written kernels instantiated in float64: FD check at 1e-6."""
    X, Y, params = problem
    loss, grads = _torch_grads(problem, dtype=torch.float64)
    assert abs(loss - _loss64([p.astype(np.float64) for p in params], X.astype(np.float64),
                              Y.astype(np.float64), eps=1e-8)) < 1e-12
    rel = _fd_relative_error(problem, grads)
    assert rel < 1e-6, rel


def test_fp32_kernels_within_float32_rounding_of_finite_differences(problem):
    """The float32 kernels against the same float64 FD: the difference is the
    float32 rounding of the forward and backward sums (~4e-6 here)."""
    _, grads = _torch_grads(problem)
    rel = _fd_relative_error(problem, grads)
    assert rel < 2e-5, rel


def test_split_bf16_gradients_close_to_fp64(problem):
    _, g32 = _torch_grads(problem, "fp32")
    _, gx3 = _torch_grads(problem, "bf16x3")
    for a, b in zip(g32, gx3):
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 2e-5


def test_autograd_equals_drop_in_nn_backward(problem, gpu):
    import vulkpy_gb300 as vk
    X, Y, params = problem
    _, grads = _torch_grads(problem)
    nn = vk.nn
    W1, b1, W2, b2 = params
    net = nn.Sequence([
        nn.Dense(gpu, 784, 32, w_init=lambda g, s: vk.Array(g, data=W1), b_init=lambda g, s: vk.Array(g, data=b1)),
        nn.ReLU(),
        nn.Dense(gpu, 32, 10, w_init=lambda g, s: vk.Array(g, data=W2), b_init=lambda g, s: vk.Array(g, data=b2)),
    ], nn.SoftmaxCrossEntropyLoss())
    out = net._forward(vk.Array(gpu, data=X))
    net.loss(out, vk.Array(gpu, data=Y))
    net._zero_grad()
    net._backward()
    mine = [np.asarray(net.L[0].w.grad), np.asarray(net.L[0].b.grad), np.asarray(net.L[2].w.grad),
            np.asarray(net.L[2].b.grad)]
    for a, b in zip(grads, mine):
        np.testing.assert_array_equal(a, b)
