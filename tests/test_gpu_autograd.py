"""Hand-written backward kernels behind torch.autograd.Function:
  * against float64 central finite differences (h = 1e-6) of the same
    network computed in numpy float64, relative error of the sampled
    gradient <= 1e-6, for Dense with ReLU / Sigmoid (fused and standalone),
    Softmax (exact backward), every loss (cross entropy, softmax cross
    entropy, MSE, Huber) and a MixLoss, including a 784 -> 32 -> 32 -> 10
    copy of the differentiable-MLP workload (Dense, ReLU, Dense, Sigmoid,
    Dense, softmax cross entropy);
  * the float32 kernels within float32 rounding (2e-5) of the same FD;
  * against this package's drop-in nn backward (vulkpy's semantics): equal
    bit for bit, in the reference-compatible variants;
  * against the reference's own nn backward (tests/golden, generated by
    vulkpy's Python): rtol 2e-6.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import scenarios  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "golden.npz"))
DEV = "cuda:0"
EPS_CE = float(np.float32(1e-8))


# ---------------------------------------------------------------- float64 models
def _softmax64(z):
    z = z - z.max(1, keepdims=True)
    e = np.exp(z)
    return e / e.sum(1, keepdims=True)


def _sigmoid64(z):
    return 1.0 / (1.0 + np.exp(-z))


def _loss_value64(kind, x, y, fd=False):
    """Mean over rows of the per-row loss, float64 (losses.py:40-458).  The
    softmax cross entropy forward takes log(p + 1e-8) (nn_cross_entropy.comp)
    while its backward is p - y (losses.py:229-249), the exact gradient of
    the loss without the 1e-8: finite differences (``fd``) are taken of that
    one.  Cross entropy's backward -y / (x + 1e-8) is the exact gradient of
    its forward, 1e-8 included."""
    if kind == "ce":
        rows = (-y * np.log(x + EPS_CE)).sum(1)
    elif kind == "sce":
        rows = (-y * np.log(_softmax64(x) + (0.0 if fd else EPS_CE))).sum(1)
    elif kind == "mse":
        rows = ((y - x) ** 2).sum(1)
    else:  # huber
        a = np.abs(y - x)
        rows = (0.5 * np.minimum(a, a * a)).sum(1)
    return rows.mean()


ACT64 = {"relu": lambda z: np.maximum(z, 0.0), "sigmoid": _sigmoid64, None: lambda z: z}


def _forward64(layers, params, X):
    """layers: list of ("dense", act) / ("relu",) / ("sigmoid",) / ("softmax",)."""
    h = X
    k = 0
    for spec in layers:
        if spec[0] == "dense":
            W, b = params[k], params[k + 1]
            k += 2
            h = ACT64[spec[1]](h @ W.T + b)
        elif spec[0] == "softmax":
            h = _softmax64(h)
        else:
            h = ACT64[spec[0]](h)
    return h


def _objective64(layers, loss_spec, params, X, Y, fd=False):
    out = _forward64(layers, params, X)
    return sum(c * _loss_value64(kind, out, Y, fd) for c, kind in loss_spec)


# ---------------------------------------------------------------- device models
def _run_torch(layers, loss_spec, params, X, Y, dtype, precision="fp32", huber_grad="exact", softmax_grad="exact"):
    import vulkpy_gb300.autograd as A
    t = [torch.tensor(p, device=DEV, dtype=dtype, requires_grad=True) for p in params]
    h = torch.tensor(X, device=DEV, dtype=dtype)
    y = torch.tensor(Y, device=DEV, dtype=dtype)
    k = 0
    for spec in layers:
        if spec[0] == "dense":
            h = A.dense(h, t[k], t[k + 1], act=spec[1], precision=precision)
            k += 2
        elif spec[0] == "softmax":
            h = A.softmax(h, grad=softmax_grad)
        elif spec[0] == "relu":
            h = A.relu(h)
        else:
            h = A.sigmoid(h)
    if len(loss_spec) == 1 and loss_spec[0][0] == 1.0:
        kind = loss_spec[0][1]
        fn = {"ce": A.cross_entropy, "sce": A.softmax_cross_entropy, "mse": A.mse}.get(kind)
        loss = A.huber(h, y, grad=huber_grad) if kind == "huber" else fn(h, y)
    else:
        loss = A.mix(loss_spec, h, y, huber_grad=huber_grad)
    loss.backward()
    torch.cuda.synchronize()
    return float(loss.detach()), [p.grad.cpu().numpy() for p in t]


def _make_params(rng, dims):
    params = []
    for i, o in zip(dims[:-1], dims[1:]):
        params.append((rng.standard_normal((o, i)) * np.sqrt(2 / i)).astype(np.float32))
        params.append((rng.standard_normal(o) * 0.1).astype(np.float32))
    return params


def _fd_relative_error(layers, loss_spec, params, X, Y, grads, samples=30, seed=2):
    p64 = [p.astype(np.float64) for p in params]
    X64, Y64 = X.astype(np.float64), Y.astype(np.float64)
    rng = np.random.default_rng(seed)
    h = 1e-6
    ours, fd = [], []
    for k, p in enumerate(p64):
        idx = rng.choice(p.size, size=min(p.size, samples), replace=False)
        for i in idx:
            plus = [q.copy() for q in p64]
            minus = [q.copy() for q in p64]
            plus[k].flat[i] += h
            minus[k].flat[i] -= h
            fd.append((_objective64(layers, loss_spec, plus, X64, Y64, fd=True)
                       - _objective64(layers, loss_spec, minus, X64, Y64, fd=True)) / (2 * h))
            ours.append(grads[k].flat[i])
    ours, fd = np.array(ours), np.array(fd)
    return np.linalg.norm(ours - fd) / np.linalg.norm(fd)


# Networks: (name, layers, dims, loss_spec, batch, target kind)
NETS = [
    ("relu_sce", [("dense", "relu"), ("dense", None)], [784, 32, 10], [(1.0, "sce")], 64, "onehot"),
    ("c4_copy", [("dense", "relu"), ("dense", "sigmoid"), ("dense", None)], [784, 32, 32, 10], [(1.0, "sce")], 64,
     "onehot"),
    ("standalone_sigmoid_softmax_ce", [("dense", None), ("sigmoid",), ("dense", None), ("softmax",)], [20, 16, 6],
     [(1.0, "ce")], 32, "onehot"),
    ("standalone_relu_mse", [("dense", None), ("relu",), ("dense", None)], [20, 16, 5], [(1.0, "mse")], 32,
     "normal"),
    ("huber", [("dense", "relu"), ("dense", None)], [20, 16, 5], [(1.0, "huber")], 32, "normal"),
    ("mix_mse_huber", [("dense", "sigmoid"), ("dense", None)], [20, 16, 5], [(0.3, "mse"), (0.7, "huber")], 32,
     "normal"),
    ("mix_sce_mse", [("dense", "relu"), ("dense", None)], [20, 16, 5], [(0.6, "sce"), (0.4, "mse")], 32,
     "onehot"),
]


def _problem(dims, batch, target, seed=1):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((batch, dims[0])).astype(np.float32)
    if target == "onehot":
        Y = np.eye(dims[-1], dtype=np.float32)[rng.integers(0, dims[-1], batch)]
    else:
        Y = (rng.standard_normal((batch, dims[-1])) * 2.0).astype(np.float32)
    return X, Y, _make_params(rng, dims)


@pytest.mark.parametrize("name,layers,dims,loss_spec,batch,target", NETS, ids=[n[0] for n in NETS])
def test_fp64_kernels_match_fp64_finite_differences(name, layers, dims, loss_spec, batch, target):
    """The hand-written kernels instantiated in float64: loss equal to the
    numpy float64 model, FD check of the gradients at 1e-6."""
    X, Y, params = _problem(dims, batch, target)
    loss, grads = _run_torch(layers, loss_spec, params, X, Y, torch.float64)
    ref = _objective64(layers, loss_spec, [p.astype(np.float64) for p in params], X.astype(np.float64),
                       Y.astype(np.float64))
    assert abs(loss - ref) <= 1e-12 * max(1.0, abs(ref))
    rel = _fd_relative_error(layers, loss_spec, params, X, Y, grads)
    assert rel < 1e-6, rel


@pytest.mark.parametrize("name,layers,dims,loss_spec,batch,target", NETS[:4], ids=[n[0] for n in NETS[:4]])
def test_fp32_kernels_within_float32_rounding_of_finite_differences(name, layers, dims, loss_spec, batch, target):
    """The float32 kernels against the same float64 FD: the difference is the
    float32 rounding of the forward and backward sums."""
    X, Y, params = _problem(dims, batch, target)
    _, grads = _run_torch(layers, loss_spec, params, X, Y, torch.float32)
    rel = _fd_relative_error(layers, loss_spec, params, X, Y, grads)
    assert rel < 2e-5, rel


def test_split_bf16_gradients_close_to_fp64():
    name, layers, dims, loss_spec, batch, target = NETS[1]
    X, Y, params = _problem(dims, batch, target)
    _, g32 = _run_torch(layers, loss_spec, params, X, Y, torch.float32, "fp32")
    _, gx3 = _run_torch(layers, loss_spec, params, X, Y, torch.float32, "bf16x3")
    for a, b in zip(g32, gx3):
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 2e-5


def test_autograd_equals_drop_in_nn_backward(gpu):
    """Dense + ReLU + Dense + Sigmoid + Dense + softmax cross entropy: the
    autograd Functions and the drop-in Sequence backward give the same
    gradients bit for bit."""
    import vulkpy_gb300 as vk
    name, layers, dims, loss_spec, batch, target = NETS[1]
    X, Y, params = _problem(dims, batch, target)
    _, grads = _run_torch(layers, loss_spec, params, X, Y, torch.float32)
    nn = vk.nn

    def dense(i, o, k):
        W, b = params[2 * k], params[2 * k + 1]
        return nn.Dense(gpu, i, o, w_init=lambda g, s: vk.Array(g, data=W), b_init=lambda g, s: vk.Array(g, data=b))

    net = nn.Sequence([dense(784, 32, 0), nn.ReLU(), dense(32, 32, 1), nn.Sigmoid(), dense(32, 10, 2)],
                      nn.SoftmaxCrossEntropyLoss())
    out = net._forward(vk.Array(gpu, data=X))
    net.loss(out, vk.Array(gpu, data=Y))
    net._zero_grad()
    net._backward()
    mine = []
    for li in (0, 2, 4):
        mine += [np.asarray(net.L[li].w.grad), np.asarray(net.L[li].b.grad)]
    for a, b in zip(grads, mine):
        np.testing.assert_array_equal(a, b)


# ---------------------------------------------------------------- per-Function checks
def _fn_grad(fn, x, *rest, dtype=torch.float32, upstream=None):
    xt = torch.tensor(x, device=DEV, dtype=dtype, requires_grad=True)
    rt = [torch.tensor(r, device=DEV, dtype=dtype) for r in rest]
    out = fn(xt, *rt)
    if upstream is None:
        out.backward()
    else:
        out.backward(torch.tensor(upstream, device=DEV, dtype=dtype))
    torch.cuda.synchronize()
    return out.detach().cpu().numpy(), xt.grad.cpu().numpy()


def test_functions_equal_drop_in_layers_and_losses(gpu):
    """Each Function in its reference-compatible variant against the drop-in
    layer's / loss's backward on the same inputs: bit for bit."""
    import vulkpy_gb300 as vk
    import vulkpy_gb300.autograd as A
    nn = vk.nn
    z, dy, prob, onehot, pred, target = scenarios.backward_suite_inputs()
    for name, layer, fn in (("relu", nn.ReLU(), A.relu), ("sigmoid", nn.Sigmoid(), A.sigmoid),
                            ("softmax", nn.Softmax(), lambda x: A.softmax(x, grad="vulkpy"))):
        y_ref = np.asarray(layer(vk.Array(gpu, data=z)))
        dx_ref = np.asarray(layer.backward(vk.Array(gpu, data=dy)))
        y, dx = _fn_grad(fn, z, upstream=dy)
        np.testing.assert_array_equal(y, y_ref, err_msg=name)
        np.testing.assert_array_equal(dx, dx_ref, err_msg=name)
    cases = (("ce", nn.CrossEntropyLoss(), A.cross_entropy, prob, onehot),
             ("sce", nn.SoftmaxCrossEntropyLoss(), A.softmax_cross_entropy, z, onehot),
             ("mse", nn.MSELoss(), A.mse, pred, target),
             ("huber", nn.HuberLoss(), lambda x, y: A.huber(x, y, grad="vulkpy"), pred, target),
             ("mix", nn.losses.MixLoss([(0.3, nn.MSELoss()), (0.7, nn.HuberLoss())]),
              lambda x, y: A.mix([(0.3, "mse"), (0.7, "huber")], x, y, huber_grad="vulkpy"), pred, target))
    for name, loss, fn, x, y in cases:
        L_ref = np.asarray(loss(vk.Array(gpu, data=x), vk.Array(gpu, data=y)))
        dx_ref = np.asarray(loss.grad())
        L, dx = _fn_grad(fn, x, y)
        np.testing.assert_array_equal(dx, dx_ref, err_msg=name)
        np.testing.assert_allclose(L, L_ref, rtol=2e-6, err_msg=name)


def test_functions_match_reference_backward_golden():
    """The same Functions against the reference's own nn backward (golden
    values generated by vulkpy's Python, scenario nn_backward_suite)."""
    import vulkpy_gb300.autograd as A
    z, dy, prob, onehot, pred, target = scenarios.backward_suite_inputs()
    G = lambda k: GOLDEN[f"nn_backward_suite/{k}"]  # noqa: E731
    tol = dict(rtol=2e-6, atol=1e-7)
    for name, fn in (("relu", A.relu), ("sigmoid", A.sigmoid), ("softmax", lambda x: A.softmax(x, grad="vulkpy"))):
        y, dx = _fn_grad(fn, z, upstream=dy)
        np.testing.assert_allclose(y, G(f"{name}_y"), err_msg=name, **tol)
        np.testing.assert_allclose(dx, G(f"{name}_dx"), err_msg=name, **tol)
    for name, fn, x, y in (("ce", A.cross_entropy, prob, onehot), ("sce", A.softmax_cross_entropy, z, onehot),
                           ("mse", A.mse, pred, target), ("huber", lambda a, b: A.huber(a, b, grad="vulkpy"), pred,
                                                          target),
                           ("mix", lambda a, b: A.mix([(0.3, "mse"), (0.7, "huber")], a, b, huber_grad="vulkpy"),
                            pred, target)):
        L, dx = _fn_grad(fn, x, y)
        np.testing.assert_allclose(dx, G(f"{name}_dx"), err_msg=name, **tol)
        np.testing.assert_allclose(L, G(f"{name}_loss"), rtol=2e-6, err_msg=name)


def test_exact_and_reference_gradients_differ_only_where_documented():
    """Softmax: the exact backward differs from the diagonal form; Huber:
    exact and clamp agree where |x - y| <= 1 and differ by a factor 2 beyond."""
    import vulkpy_gb300.autograd as A
    z, dy, prob, onehot, pred, target = scenarios.backward_suite_inputs()
    _, d_exact = _fn_grad(lambda x: A.softmax(x), z, upstream=dy)
    _, d_diag = _fn_grad(lambda x: A.softmax(x, grad="vulkpy"), z, upstream=dy)
    s = _softmax64(z.astype(np.float64))
    jvp = s * (dy - (dy * s).sum(1, keepdims=True))
    np.testing.assert_allclose(d_exact, jvp, rtol=1e-5, atol=1e-6)
    assert np.abs(d_exact - d_diag).max() > 1e-3
    _, h_exact = _fn_grad(lambda x, y: A.huber(x, y), pred, target)
    _, h_ref = _fn_grad(lambda x, y: A.huber(x, y, grad="vulkpy"), pred, target)
    d = pred.astype(np.float64) - target
    inside = np.abs(d) <= 1
    assert inside.any() and (~inside).any()
    np.testing.assert_array_equal(h_exact[inside], h_ref[inside])
    np.testing.assert_allclose(h_exact[~inside] * 2, h_ref[~inside], rtol=1e-6)
