"""The training loop of the reference's classification example
(example/02-nn.py:60-107: 4-128-128-3 Dense/ReLU/Softmax, CrossEntropyLoss
with reduce="sum", Adam, batch 32, shuffled every epoch) on a synthetic
Iris-shaped data set (150 rows, 4 features, 3 classes, 120/30 split).

Three ways to run it must agree bit for bit when they draw the same order:
  * host loop: shuffle on the host, upload each batch (the example's way),
    with the order taken from the oracle's permutation of the same seed;
  * device loop: ``nn.minibatches`` with the device permutation;
  * the device loop's epoch captured once in a CUDA graph and replayed."""
import numpy as np
import pytest

from oracle.ops import Xoshiro128pp as OracleXo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


def iris_like(seed=0):
    rng = np.random.default_rng(seed)
    means = rng.uniform(1.0, 7.0, size=(3, 4))
    x = np.concatenate([rng.normal(means[c], 0.45, size=(50, 4)) for c in range(3)]).astype(np.float32)
    y = np.repeat(np.arange(3), 50)
    order = rng.permutation(150)
    x, y = x[order], y[order]
    onehot = np.identity(3, dtype=np.float32)[y]
    return x[:120], onehot[:120], x[120:], onehot[120:]


def make_net(vk, gpu):
    nn = vk.nn
    opt = nn.Adam(gpu, lr=1e-3)
    return nn.Sequence([
        nn.Dense(gpu, 4, 128, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 4, seed=1)),
        nn.ReLU(),
        nn.Dense(gpu, 128, 128, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 128, seed=2)),
        nn.ReLU(),
        nn.Dense(gpu, 128, 3, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 128, seed=3)),
        nn.Softmax(),
    ], nn.CrossEntropyLoss(reduce="sum"))


def weights(net):
    out = [np.asarray(p.value).copy() for layer in net.L if isinstance(layer, vk_dense())
           for p in (layer.w, layer.b)]
    assert len(out) == 6
    return out


def vk_dense():
    from vulkpy_gb300.nn import Dense
    return Dense


def test_device_loop_matches_host_loop(gpu, vk):
    tx, ty, vx, vy = iris_like()
    B, epochs, seed = 32, 4, 9

    # host loop, order from the oracle's copy of the device permutation
    net_h = make_net(vk, gpu)
    o = OracleXo(seed, 64)
    host_losses = []
    for _ in range(epochs):
        perm = o.permutation(120)
        total = vk.Array(gpu, shape=(1,))
        total[:] = 0
        for s in range(0, 120, B):
            rows = perm[s:s + B]
            _, loss = net_h.train(vk.Array(gpu, data=tx[rows]), vk.Array(gpu, data=ty[rows]))
            total += loss
        host_losses.append(float(np.asarray(total)[0]))

    # device loop
    net_d = make_net(vk, gpu)
    r = vk.random.Xoshiro128pp(gpu, seed=seed)
    X, Y = vk.Array(gpu, data=tx), vk.Array(gpu, data=ty)
    dev_losses = []
    for _ in range(epochs):
        total = vk.Array(gpu, shape=(1,))
        total[:] = 0
        for x, y in vk.nn.minibatches(X, Y, B, rng=r):
            _, loss = net_d.train(x, y)
            total += loss
        dev_losses.append(float(np.asarray(total)[0]))

    assert host_losses == dev_losses
    for a, b in zip(weights(net_h), weights(net_d)):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(r.state().reshape(-1), o.state)
    assert gpu.check_errors() == 0


def test_graph_epoch_matches_eager_and_learns(gpu, vk):
    tx, ty, vx, vy = iris_like()
    B, seed = 32, 4
    X, Y = vk.Array(gpu, data=tx), vk.Array(gpu, data=ty)
    VX = vk.Array(gpu, data=vx)

    def epoch(net, r):
        total = vk.zeros(gpu, shape=(1,))
        for x, y in vk.nn.minibatches(X, Y, B, rng=r):
            _, loss = net.train(x, y)
            total += loss
        cls = net.predict(VX).argmax(axis=1)
        return total, cls

    # eager reference run
    net_e, r_e = make_net(vk, gpu), vk.random.Xoshiro128pp(gpu, seed=seed)
    eager = []
    for _ in range(30):
        total, cls = epoch(net_e, r_e)
        eager.append((float(np.asarray(total)[0]), np.asarray(cls).copy()))

    # first epoch eager, then one captured epoch replayed
    net_g, r_g = make_net(vk, gpu), vk.random.Xoshiro128pp(gpu, seed=seed)
    total, cls = epoch(net_g, r_g)
    got = [(float(np.asarray(total)[0]), np.asarray(cls).copy())]
    g = vk.graph.Graph(gpu)
    with g:
        total, cls = epoch(net_g, r_g)
    for _ in range(29):
        g.launch()
        got.append((float(np.asarray(total)[0]), np.asarray(cls).copy()))

    for (le, ce), (lg, cg) in zip(eager, got):
        assert le == lg
        np.testing.assert_array_equal(ce, cg)
    for a, b in zip(weights(net_e), weights(net_g)):
        np.testing.assert_array_equal(a, b)
    # the synthetic classes are well separated: the net learns them
    acc = float(np.mean(got[-1][1] == np.argmax(vy, axis=1)))
    assert acc >= 0.9, acc
    assert got[-1][0] < got[0][0]
