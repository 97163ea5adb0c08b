"""nn kernels on the GPU against float32 / float64 restatements of the
reference's layer, loss and optimizer math (vulkpy/nn/*.py).

Optimizers are bit-exact: the fused kernels reproduce the reference's chain
of float32 array ops (optimizers.py:39-52, 120-139, 221-253), restated here
op by op in numpy float32 (no fused multiply-add)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
f32 = np.float32


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


def adam_reference(value, grad, m, v, b1t, b2t, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    m = (m * f32(beta1)).astype(f32)
    m = (m + (f32(1 - beta1) * grad).astype(f32)).astype(f32)
    v = (v * f32(beta2)).astype(f32)
    v = (v + (f32(1 - beta2) * (grad * grad).astype(f32)).astype(f32)).astype(f32)
    b1t *= beta1
    b2t *= beta2
    mhat = (m / f32(1 - b1t)).astype(f32)
    vhat = (v / f32(1 - b2t)).astype(f32)
    vhat = np.sqrt(vhat).astype(f32)
    vhat = (vhat + f32(eps)).astype(f32)
    mhat = (mhat * f32(-lr)).astype(f32)
    mhat = (mhat / vhat).astype(f32)
    return (value + mhat).astype(f32), m, v, b1t, b2t


def test_adam_bit_exact_over_steps(gpu, vk):
    rng = np.random.default_rng(0)
    n = 100003
    value = rng.standard_normal(n).astype(f32)
    p = vk.nn.Parameter(gpu, (n,), opt=vk.nn.Adam(gpu, lr=1e-3), initializer=lambda g, s: vk.Array(g, data=value))
    m = np.zeros(n, f32); v = np.zeros(n, f32); b1t = b2t = 1.0
    val = value.copy()
    for step in range(4):
        grad = rng.standard_normal(n).astype(f32) * f32(10 ** (step - 2))
        p.grad[:] = 0.0
        p.add_grad(vk.Array(gpu, data=grad))
        p.update()
        val, m, v, b1t, b2t = adam_reference(val, grad, m, v, b1t, b2t)
        np.testing.assert_array_equal(np.asarray(p.value), val)
        np.testing.assert_array_equal(np.asarray(p.opt_state.m), m)
        np.testing.assert_array_equal(np.asarray(p.opt_state.v), v)


def test_sgd_and_adagrad_bit_exact(gpu, vk):
    rng = np.random.default_rng(1)
    n = 4099
    g = rng.standard_normal(n).astype(f32)
    v0 = rng.standard_normal(n).astype(f32)
    p = vk.nn.Parameter(gpu, (n,), opt=vk.nn.SGD(0.01), initializer=lambda gg, s: vk.Array(gg, data=v0))
    p.add_grad(vk.Array(gpu, data=g))
    p.update()
    np.testing.assert_array_equal(np.asarray(p.value), (v0 + (f32(-0.01) * g).astype(f32)).astype(f32))
    q = vk.nn.Parameter(gpu, (n,), opt=vk.nn.AdaGrad(gpu, lr=0.05, tau=0.1), initializer=lambda gg, s: vk.Array(gg, data=v0))
    q.add_grad(vk.Array(gpu, data=g))
    q.update()
    h = (np.full(n, f32(0.1)) + (g * g).astype(f32)).astype(f32)
    r = (g / (np.sqrt(h).astype(f32) + f32(1e-8)).astype(f32)).astype(f32)
    r = (r * f32(-0.05)).astype(f32)
    np.testing.assert_array_equal(np.asarray(q.value), (v0 + r).astype(f32))


@pytest.mark.parametrize("B,I,Out", [(1, 1, 1), (2, 3, 4), (33, 65, 17), (256, 784, 1024), (7, 1024, 10)])
def test_dense_forward_backward(gpu, vk, B, I, Out):
    rng = np.random.default_rng(B * I + Out)
    x = rng.standard_normal((B, I)).astype(f32)
    W = rng.standard_normal((Out, I)).astype(f32) * f32(0.1)
    b = rng.standard_normal(Out).astype(f32)
    dy = rng.standard_normal((B, Out)).astype(f32)
    d = vk.nn.Dense(gpu, I, Out, w_init=lambda g, s: vk.Array(g, data=W), b_init=lambda g, s: vk.Array(g, data=b))
    X = vk.Array(gpu, data=x)
    y = np.asarray(d(X))
    x64, W64 = x.astype(np.float64), W.astype(np.float64)
    y64 = x64 @ W64.T + b
    np.testing.assert_allclose(y, y64, rtol=1e-5, atol=1e-5 * np.sqrt(I))
    dx = np.asarray(d.backward(vk.Array(gpu, data=dy)))
    np.testing.assert_allclose(dx, dy.astype(np.float64) @ W64, rtol=1e-5, atol=1e-5 * np.sqrt(Out))
    np.testing.assert_allclose(np.asarray(d.w.grad), dy.astype(np.float64).T @ x64, rtol=1e-5,
                               atol=1e-5 * np.sqrt(B))
    np.testing.assert_allclose(np.asarray(d.b.grad), dy.astype(np.float64).sum(0), rtol=1e-5, atol=1e-5 * np.sqrt(B))


def test_softmax_cross_entropy_rows(gpu, vk):
    rng = np.random.default_rng(2)
    x = rng.standard_normal((300, 10)).astype(f32) * 3
    y = np.eye(10, dtype=f32)[rng.integers(0, 10, 300)]
    sce = vk.nn.SoftmaxCrossEntropyLoss()
    L = np.asarray(sce(vk.Array(gpu, data=x), vk.Array(gpu, data=y)))
    x64 = x.astype(np.float64)
    p = np.exp(x64 - x64.max(1, keepdims=True))
    p /= p.sum(1, keepdims=True)
    Lr = (-y * np.log(p + 1e-8)).sum(1).mean()
    np.testing.assert_allclose(L, [Lr], rtol=1e-5)
    np.testing.assert_allclose(np.asarray(sce.grad()), (p - y) / 300, rtol=1e-5, atol=1e-7)
    sm = vk.nn.Softmax()
    np.testing.assert_allclose(np.asarray(sm(vk.Array(gpu, data=x))), p, rtol=1e-5, atol=1e-7)


def _mlp(vk, gpu, fuse=True, seed=3):
    nn = vk.nn
    opt = nn.Adam(gpu, lr=1e-2)
    return nn.Sequence([
        nn.Dense(gpu, 20, 16, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 20, seed=seed)),
        nn.ReLU(),
        nn.Dense(gpu, 16, 12, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 16, seed=seed + 1)),
        nn.Sigmoid(),
        nn.Dense(gpu, 12, 5, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 12, seed=seed + 2)),
    ], nn.SoftmaxCrossEntropyLoss(), fuse=fuse)


def _params(net):
    return [np.asarray(p).copy() for L in net.L if hasattr(L, "w") for p in (L.w.value, L.b.value)]


@pytest.mark.parametrize("batch", [32, 300])
@pytest.mark.parametrize("prec", ["fp32", "bf16x3"])
def test_fused_sequence_and_graph_replay_are_bit_identical(gpu, vk, prec, batch):
    """Dense+activation fusion (forward epilogue; backward activation
    derivative + bias sum in one kernel, over one partial or a full and a
    partial 256-row chunk) and CUDA-graph replay change how many kernels
    run, not the float32 results: parameters and losses match eager,
    unfused steps bit for bit."""
    rng = np.random.default_rng(0)
    X = rng.standard_normal((batch, 20)).astype(f32)
    Y = np.eye(5, dtype=f32)[rng.integers(0, 5, batch)]
    old = gpu.matmul_precision
    gpu.matmul_precision = prec
    try:
        ref = _mlp(vk, gpu, fuse=False)
        fused = _mlp(vk, gpu, fuse=True)
        graphed = _mlp(vk, gpu, fuse=True)
        x, y = vk.Array(gpu, data=X), vk.Array(gpu, data=Y)
        losses = []
        for _ in range(4):
            _, l = ref.train(x, y)
            losses.append(np.asarray(l).copy())
        for i in range(4):
            _, l = fused.train(x, y)
            np.testing.assert_array_equal(np.asarray(l), losses[i])
        graphed.train(x, y)
        step = graphed.compile(x, y)
        for i in range(1, 4):
            _, l = step()
            np.testing.assert_array_equal(np.asarray(l), losses[i])
        for a, b, c in zip(_params(ref), _params(fused), _params(graphed)):
            np.testing.assert_array_equal(a, b)
            np.testing.assert_array_equal(a, c)
    finally:
        gpu.matmul_precision = old


def test_graph_capture_replays_ops(gpu, vk):
    x = vk.Array(gpu, data=np.arange(8, dtype=f32))
    g = vk.graph.Graph(gpu)
    with g:
        y = (x * 2.0).exp()
        s = y.sum()
    g.launch()
    np.testing.assert_allclose(np.asarray(y), np.exp(np.arange(8) * 2.0), rtol=1e-6)
    x[:] = 1.0                     # host write, uploaded by launch(flush=...)
    g.launch(flush=[x])
    np.testing.assert_allclose(np.asarray(y), np.full(8, np.exp(2.0)), rtol=1e-6)
    np.testing.assert_allclose(np.asarray(s), [8 * np.exp(2.0)], rtol=1e-6)


def test_branches_in_a_graph_match_sequential_eager(gpu, vk):
    """Several independent models trained in parallel graph branches give the
    same parameters as training them one after another eagerly."""
    rng = np.random.default_rng(5)
    shapes = [(17, 40, 3, 9), (64, 33, 8, 1), (30, 129, 5, 31)]
    def build():
        nets = []
        for k, (i, h, o, b) in enumerate(shapes):
            opt = vk.nn.SGD(lr=1e-2)
            nets.append(vk.nn.Sequence([
                vk.nn.Dense(gpu, i, h, w_opt=opt, b_opt=opt, w_init=vk.nn.HeNormal(gpu, i, seed=k)),
                vk.nn.ReLU(),
                vk.nn.Dense(gpu, h, o, w_opt=opt, b_opt=opt, w_init=vk.nn.HeNormal(gpu, h, seed=10 + k)),
            ], vk.nn.MSELoss()))
        return nets
    data = [(vk.Array(gpu, data=rng.standard_normal((b, i)).astype(f32)),
             vk.Array(gpu, data=rng.standard_normal((b, o)).astype(f32))) for i, h, o, b in shapes]
    ref, par = build(), build()
    for _ in range(3):
        for net, (x, y) in zip(ref, data):
            net.train(x, y)
    for net, (x, y) in zip(par, data):
        net.train(x, y)
    g = vk.graph.Graph(gpu)
    with g:
        for net, (x, y) in zip(par, data):
            with gpu.branch():
                net.train(x, y)
    g.launch()
    g.launch()
    for a, b in zip(ref, par):
        for pa, pb in zip(_params(a), _params(b)):
            np.testing.assert_array_equal(pa, pb)
    # eager branches (no graph) too
    eager = build()
    for _ in range(3):
        for net, (x, y) in zip(eager, data):
            with gpu.branch():
                net.train(x, y)
    for a, b in zip(ref, eager):
        for pa, pb in zip(_params(a), _params(b)):
            np.testing.assert_array_equal(pa, pb)


@pytest.mark.parametrize("hidden", [16, 130])
@pytest.mark.parametrize("optname", ["adam", "sgd"])
def test_grouped_parameter_update_matches_per_parameter(gpu, vk, optname, hidden):
    """A Sequence whose parameters share one optimizer zeroes every gradient
    and updates every parameter in one launch each; a copy whose layers have
    their own optimizer objects (same hyperparameters) takes the
    per-parameter path.  Parameters, moments and the device-side Adam powers
    match bit for bit, eager and replayed from a captured step.  Hidden width
    130 gives a 64 x 130 weight (two full 4096-element chunks, the 128-bit
    path, plus a ragged tail)."""
    nn = vk.nn
    rng = np.random.default_rng(4)
    n_in = 12 if hidden == 16 else 64
    X = rng.standard_normal((24, n_in)).astype(f32)
    Y = np.eye(3, dtype=f32)[rng.integers(0, 3, 24)]

    def make(shared):
        mk = (lambda: nn.Adam(gpu, lr=1e-2)) if optname == "adam" else (lambda: nn.SGD(lr=1e-2))
        o = mk()
        opts = [o if shared else mk() for _ in range(4)]
        return nn.Sequence([
            nn.Dense(gpu, n_in, hidden, w_opt=opts[0], b_opt=opts[1], w_init=nn.HeNormal(gpu, n_in, seed=3)),
            nn.ReLU(),
            nn.Dense(gpu, hidden, 3, w_opt=opts[2], b_opt=opts[3], w_init=nn.HeNormal(gpu, hidden, seed=4)),
        ], nn.SoftmaxCrossEntropyLoss())

    per, grouped, graphed = make(False), make(True), make(True)
    assert per._update_grouped(per._params()) is False   # separate optimizers: per-parameter path
    x, y = vk.Array(gpu, data=X), vk.Array(gpu, data=Y)
    for _ in range(3):
        per.train(x, y)
        grouped.train(x, y)
    graphed.train(x, y)
    step = graphed.compile(x, y)
    step()
    step()
    for a, b, c in zip(_params(per), _params(grouped), _params(graphed)):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, c)
    if optname == "adam":
        for La, Lb in ((per.L[0], grouped.L[0]), (per.L[2], grouped.L[2])):
            for pa, pb in ((La.w, Lb.w), (La.b, Lb.b)):
                np.testing.assert_array_equal(np.asarray(pa.opt_state.m), np.asarray(pb.opt_state.m))
                np.testing.assert_array_equal(np.asarray(pa.opt_state.v), np.asarray(pb.opt_state.v))
                np.testing.assert_array_equal(np.asarray(pa.opt_state._powers), np.asarray(pb.opt_state._powers))
                assert pa.opt_state.beta1t == pb.opt_state.beta1t


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3"])
@pytest.mark.parametrize("B,I,Out", [(256, 1024, 1024), (256, 1024, 10), (37, 300, 130)])
def test_backward_chain_matches_backward_then_activation(gpu, vk, prec, B, I, Out):
    """Dense.backward_chain (the activation derivative below the layer in the
    input-gradient GEMM's epilogue or split-K reduction, in or outside a
    cluster) gives the bits of Dense.backward followed by the activation's
    own backward kernel, for ReLU and sigmoid, whole-K and split-K plans."""
    from vulkpy_gb300 import _lib, autotune
    from vulkpy_gb300.nn.layers import _act_backward
    rng = np.random.default_rng(B + I + Out)
    X = rng.standard_normal((B, I)).astype(f32)
    DY = rng.standard_normal((B, Out)).astype(f32)
    Yr = np.maximum(rng.standard_normal((B, I)), 0).astype(f32)
    Yr[0, :5] = [0.0, -0.0, np.nan, 1e-30, -1e-30]
    Ys = (1 / (1 + np.exp(-rng.standard_normal((B, I))))).astype(f32)
    P = {"fp32": _lib.MM_FP32, "bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}[prec]
    old = gpu.matmul_precision
    gpu.matmul_precision = prec
    try:
        d = vk.nn.Dense(gpu, I, Out)
        x = vk.Array(gpu, data=X)
        d(x)
        dy = vk.Array(gpu, data=DY)
        for splits in (0, 1, 3, 8):
            if splits:
                _lib.lib.vkc_gemm_plan_set(P, B, I, Out, splits, 128)
            for act, Yh in ((_lib.ACT_RELU, Yr), (_lib.ACT_SIGMOID, Ys)):
                y = vk.Array(gpu, data=Yh)
                for cl in (1, 0):
                    _lib.lib.vkc_set_cluster_splitk(cl)
                    got = np.asarray(d.backward_chain(dy, act, y, accumulate=False)).copy()
                    gw, gb = np.asarray(d.w.grad).copy(), np.asarray(d.b.grad).copy()
                    dx = d.backward(dy, accumulate=False)
                    ref = np.asarray(_act_backward(act, y, dx)).copy()
                    np.testing.assert_array_equal(got, ref, err_msg=str((splits, act, cl)))
                    np.testing.assert_array_equal(gw, np.asarray(d.w.grad))
                    np.testing.assert_array_equal(gb, np.asarray(d.b.grad))
    finally:
        gpu.matmul_precision = old
        _lib.lib.vkc_set_cluster_splitk(0)   # the default
        _lib.lib.vkc_gemm_tune_set(P, B, I, Out, 0)
        autotune.load_table()
    assert gpu.check_errors() == 0


@pytest.mark.parametrize("prec", ["bf16", "bf16x3"])
@pytest.mark.parametrize("dims,batch", [((784, 1024, 1024, 10), 256), ((100, 300, 130, 7), 37), ((64, 96, 64), 130),
                                        ((16, 8, 1), 5), ((16, 8, 4), 1)])
def test_dense_stack_forward_matches_layer_by_layer(gpu, vk, prec, dims, batch):
    """vkc_dense_stack_forward (each layer's split-K reduction writing the
    next layer's operand pre-pass, weights split on a side stream) gives the
    bits of vkc_dense_forward layer by layer, whole-K and split-K plans;
    shapes off the tensor-core path (N = 1, batch 1) run layer by layer."""
    import ctypes as C
    from vulkpy_gb300 import _lib, autotune
    P = {"bf16": _lib.MM_BF16, "bf16x3": _lib.MM_BF16X3}[prec]
    rng = np.random.default_rng(sum(dims) + batch)
    X = rng.standard_normal((batch, dims[0])).astype(f32)
    Ws = [(rng.standard_normal((o, i)) / np.sqrt(i)).astype(f32) for i, o in zip(dims[:-1], dims[1:])]
    bs = [rng.standard_normal(o).astype(f32) for o in dims[1:]]
    acts = [_lib.ACT_RELU, _lib.ACT_SIGMOID, _lib.ACT_NONE][:len(Ws)]
    acts[-1] = _lib.ACT_NONE
    x = vk.Array(gpu, data=X)
    w = [vk.Array(gpu, data=a) for a in Ws]
    b = [vk.Array(gpu, data=a) for a in bs]
    k = len(Ws)
    try:
        for splits in (0, 1, 3, 8):
            if splits:
                for i, o in zip(dims[:-1], dims[1:]):
                    _lib.lib.vkc_gemm_plan_set(P, batch, o, i, splits, 128)
            ys = [vk.Array(gpu, shape=(batch, o)) for o in dims[1:]]
            ptrs = lambda v: (C.c_void_p * k)(*v)
            st = _lib.lib.vkc_dense_stack_forward(
                gpu.handle, P, k, x._dptr(), batch, (C.c_int64 * (k + 1))(*dims), ptrs([a._dptr() for a in w]),
                ptrs([a._dptr() for a in b]), (C.c_int * k)(*acts), ptrs([y._buf.ptr for y in ys]))
            assert st == 0, _lib.last_error()
            inp = x
            for l in range(k):
                ys[l]._written()
                ref = vk.Array(gpu, shape=(batch, dims[l + 1]))
                assert _lib.lib.vkc_dense_forward(gpu.handle, P, inp._dptr(), w[l]._dptr(), b[l]._dptr(), ref._buf.ptr,
                                                  batch, dims[l], dims[l + 1], acts[l]) == 0
                ref._written()
                np.testing.assert_array_equal(np.asarray(ys[l]), np.asarray(ref), err_msg=str((splits, l)))
                inp = ys[l]
    finally:
        _lib.lib.vkc_gemm_tune_clear()
        autotune.load_table()
    assert gpu.check_errors() == 0
