"""
Golden scenarios: small programs written against the vulkpy API.

Each scenario is ``fn(vk) -> {name: ndarray}`` and runs unchanged on any
module with vulkpy's API.  ``make_golden.py`` runs them on the reference's
own Python (vulkpy/vkarray.py, random.py, nn/) over the oracle's fake native
module and stores the outputs in ``golden.npz``; the GPU tests run them on
``vulkpy_gb300`` and compare with the tolerance named here.

Inputs follow the reference's known-answer tests (test/test_vulkpy.py,
test/test_random.py, test/test_nn.py) and the small op suite (512x1024
uniform[-1,1) operands, seed 0).  Tolerance kinds:
  ("exact",)          bit-identical (integers, IEEE + - * /, max/min, copies)
  ("ulp", n)          within n float32 ulp of the reference output
  ("rtol", r, a)      np.testing.assert_allclose(rtol=r, atol=a)
"""
from __future__ import annotations

import numpy as np

SCENARIOS = []


def scenario(tol=("exact",)):
    def deco(fn):
        SCENARIOS.append((fn.__name__, fn, tol))
        return fn
    return deco


def A(x):
    return np.asarray(x)


# ------------------------------------------------------------ arithmetic
@scenario()
def arith_same_shape(vk):
    g = vk.GPU()
    a = vk.Array(g, data=[5, 5, 5]); b = vk.Array(g, data=[1, 1, 1]); c = vk.Array(g, data=[4, 4, 4])
    out = {"add": A(a + b), "sub": A(a - b), "mul": A(a * c), "div": A(a / c), "cascade": A(a + b + c)}
    d = vk.Array(g, data=[[1, 1], [1, 1]]); e = vk.Array(g, data=[[2, 2], [2, 2]])
    out["2d"] = A(d + e)
    x = vk.Array(g, data=[1, 1, 1]); y = vk.Array(g, data=[2, 2, 2])
    z = x + y
    out["chain"] = A(x + z)
    return out


@scenario()
def arith_inplace(vk):
    g = vk.GPU()
    out = {}
    for name, op in (("iadd", lambda a, b: a.__iadd__(b)), ("isub", lambda a, b: a.__isub__(b)),
                     ("imul", lambda a, b: a.__imul__(b)), ("idiv", lambda a, b: a.__itruediv__(b))):
        a = vk.Array(g, data=[3, 7, 2]); b = vk.Array(g, data=[2, 3, 5])
        out[name] = A(op(a, b))
    return out


@scenario()
def arith_scalar(vk):
    g = vk.GPU()
    a = vk.Array(g, data=[2.0, -3.0, 5.5])
    out = {"add": A(a + 5), "sub": A(a - 3), "mul": A(a * 3), "div": A(a / 2),
           "radd": A(3 + a), "rsub": A(4 - a), "rmul": A(7 * a), "rdiv": A(8 / a)}
    for name in ("iadd", "isub", "imul", "idiv"):
        b = vk.Array(g, data=[8.0, 3.0, -1.5])
        if name == "iadd": b += 5
        if name == "isub": b -= 1
        if name == "imul": b *= 5
        if name == "idiv": b /= 4
        out[name] = A(b)
    return out


@scenario()
def write_then_op(vk):
    g = vk.GPU()
    a = vk.Array(g, shape=(3,)); b = vk.Array(g, shape=(3,))
    a[:] = 5; b[:] = 7
    c = a + b
    b[1] = 100.0
    d = a + b
    return {"c": A(c), "d": A(d)}


@scenario()
def matmul_kat(vk):
    g = vk.GPU()
    a = vk.Array(g, data=[[1, 2], [3, 4]]); v = vk.Array(g, data=[1, 3]); w = vk.Array(g, data=[1, 2])
    return {"mm": A(a @ a), "mv": A(a @ v), "vm": A(w @ a)}


@scenario()
def reshape_kat(vk):
    g = vk.GPU()
    a = vk.Array(g, data=[1, 2, 3, 4])
    a.reshape((2, 2))
    return {"r": A(a), "shape": np.asarray(a.shape)}


@scenario()
def max_min(vk):
    g = vk.GPU()
    a = vk.Array(g, data=[1, 2, 3]); b = vk.Array(g, data=[3, 2, 1])
    out = {"max": A(a.max(b)), "min": A(a.min(b)), "max_s": A(a.max(2.0)), "min_s": A(a.min(2.0))}
    c = vk.Array(g, data=[1, 2, 3]); c.max(b, inplace=True); out["imax"] = A(c)
    d = vk.Array(g, data=[1, 2, 3]); d.min(2.0, inplace=True); out["imin_s"] = A(d)
    return out


# ------------------------------------------------------------ math
_MATH_INPUTS = {
    "abs": [-1.0, 0.0, 2.5], "sign": [-2.0, 0.0, 3.0], "sin": [0.1, 1.0, -2.0], "cos": [0.1, 1.0, -2.0],
    "tan": [0.1, 0.5, -1.0], "asin": [0.5, 0.3, -0.2], "acos": [0.5, 0.3, -0.2], "atan": [0.5, 3.0, -2.0],
    "sinh": [0.5, 1.3, -2.0], "cosh": [0.5, 1.3, -2.0], "tanh": [0.5, 1.3, -2.0],
    "asinh": [0.5, 1.3, -2.0], "acosh": [1.5, 2.3, 4.0], "atanh": [0.5, 0.3, -0.2],
    "exp": [1, 2, 3], "log": [1, 2, 3], "exp2": [1, 2, 3], "log2": [1, 2, 3], "sqrt": [1, 2, 3],
    "invsqrt": [1, 2, 3],
}


@scenario(tol=("ulp", 4))
def math_functions(vk):
    g = vk.GPU()
    out = {}
    for name, x in _MATH_INPUTS.items():
        a = vk.Array(g, data=x)
        out[name] = A(getattr(a, name)())
        b = vk.Array(g, data=x)
        getattr(b, name)(inplace=True)
        out["i" + name] = A(b)
    return out


@scenario(tol=("ulp", 4))
def pow_family(vk):
    g = vk.GPU()
    x = [1, 2, 3]; y = [1.1, 2.2, 1.4]
    a = vk.Array(g, data=x); b = vk.Array(g, data=y)
    out = {"pow": A(a ** b), "pow_s": A(a ** 2.7), "rpow": A(1.3 ** b), "sq": A(b ** 2.0)}
    c = vk.Array(g, data=x); c **= b; out["ipow"] = A(c)
    d = vk.Array(g, data=x); d **= 2.7; out["ipow_s"] = A(d)
    e = vk.Array(g, data=[[1, 2], [3, 4]]); f = vk.Array(g, data=[2, 3])
    out["pow_b"] = A(e ** f)
    return out


@scenario()
def clamp_family(vk):
    g = vk.GPU()
    x = [1.2, 3.5, 10]; lo = [3, 3, 4]; hi = [6, 6, 7]
    a = vk.Array(g, data=x); b = vk.Array(g, data=lo); c = vk.Array(g, data=hi)
    out = {"vv": A(a.clamp(b, c)), "ss": A(a.clamp(2.0, 5.0)), "sv": A(a.clamp(2.0, c)), "vs": A(a.clamp(b, 5.0))}
    d = vk.Array(g, data=x); d.clamp(b, c, inplace=True); out["ivv"] = A(d)
    e = vk.Array(g, data=x); e.clamp(2.0, 5.0, inplace=True); out["iss"] = A(e)
    m = vk.Array(g, data=[[1, 2], [3, 4]]); lo2 = vk.Array(g, data=[[2, 3]]); hi2 = vk.Array(g, data=[2, 3])
    out["b_vv"] = A(m.clamp(lo2, hi2)); out["b_vs"] = A(m.clamp(lo2, 5)); out["b_sv"] = A(m.clamp(2, hi2))
    n = vk.Array(g, data=[[1, 2], [3, 4]]); n.clamp(lo2, hi2, inplace=True); out["ib_vv"] = A(n)
    return out


# ------------------------------------------------------------ reductions
@scenario(tol=("rtol", 1e-6, 1e-6))
def reductions_small(vk):
    g = vk.GPU()
    out = {}
    x7 = np.arange(2 * 3 * 4 * 2 * 2 * 4 * 3, dtype=np.float64).reshape(2, 3, 4, 2, 2, 4, 3) % 7 - 3
    for red in ("sum", "prod", "maximum", "minimum", "mean"):
        a = vk.Array(g, data=[1, 2, 3])
        out[red] = A(getattr(a, red)())
        out[red + "_keep"] = A(getattr(vk.Array(g, data=np.ones((2, 2))), red)(keepdims=True))
        out[red + "_large"] = A(getattr(vk.Array(g, data=np.arange(65) % 5 + 1.0), red)())
        out[red + "_axis0"] = A(getattr(vk.Array(g, data=[1, 2, 3]), red)(axis=0))
        out[red + "_axis_keep"] = A(getattr(vk.Array(g, data=np.ones((2, 2))), red)(axis=0, keepdims=True))
        out[red + "_axis1"] = A(getattr(vk.Array(g, data=[[1, 2], [3, 4]]), red)(axis=1))
        out[red + "_multi"] = A(getattr(vk.Array(g, data=np.ones((2, 3, 4, 2)) * 1.5), red)(axis=(1, 2)))
        src = x7 if red != "prod" else (x7 % 2 + 1) * 0.5 + 0.5
        out[red + "_multi7"] = A(getattr(vk.Array(g, data=src), red)(axis=(1, 2, 5)))
        out[red + "_rebroadcast"] = A(getattr(vk.Array(g, data=[[1, 2], [3, 4]]), red)(axis=0, rebroadcast=True))
    return out


# ------------------------------------------------------------ broadcast / gather
@scenario()
def broadcast_family(vk):
    g = vk.GPU()
    out = {}
    out["to_3d"] = A(vk.Array(g, data=np.ones((1, 2, 2))).broadcast_to((3, 2, 2)))
    out["to_unique"] = A(vk.Array(g, data=[1, 2, 3]).broadcast_to((2, 3)))
    out["to_newdim"] = A(vk.Array(g, data=np.arange(4.0).reshape(2, 2)).broadcast_to((3, 2, 2)))
    _a = np.arange(4).reshape((1, 2, 2)); _b = np.arange(4).reshape((2, 2, 1)) + 0.5
    a = vk.Array(g, data=_a); b = vk.Array(g, data=_b)
    out["both_add"] = A(a + b); out["both_sub"] = A(a - b); out["both_mul"] = A(a * b)
    out["both_div"] = A(a / b); out["both_max"] = A(a.max(b)); out["both_min"] = A(a.min(b))
    c = vk.Array(g, data=np.ones((2, 1)) * 3); d = vk.Array(g, data=np.arange(4.0).reshape(2, 2))
    out["col"] = A(c + d)
    e = vk.Array(g, data=[1.0, 2.0])
    out["newaxis"] = A(e * d)
    # in-place broadcast where the reference's ndim bookkeeping holds (shape[0] == ndim)
    f = vk.Array(g, data=[[1, 2], [3, 4]]); f **= vk.Array(g, data=[[2, 3]]); out["ipow_row"] = A(f)
    h = vk.Array(g, data=[[1, 2], [3, 4]]); h += vk.Array(g, data=[10, 20]); out["iadd_new"] = A(h)
    k = vk.Array(g, data=[[1, 2], [3, 4]]); k -= vk.Array(g, data=[[5], [6]]); out["isub_col"] = A(k)
    return out


@scenario()
def gather_family(vk):
    g = vk.GPU()
    _a = np.arange(8).reshape((2, 2, 2))
    a = vk.Array(g, data=_a)
    out = {"flat": A(a.gather(vk.U32Array(g, data=[0, 1, 6, 7])))}
    out["flat2d"] = A(a.gather(vk.U32Array(g, data=[[0, 1], [6, 7]])))
    b = vk.Array(g, data=np.arange(30).reshape((3, 2, 5)))
    out["axis1"] = A(b.gather(vk.U32Array(g, data=[[0, 1], [1, 1]]), axis=1))
    out["axis0"] = A(b.gather(vk.U32Array(g, data=[2, 0]), axis=0))
    out["axis2"] = A(b.gather(vk.U32Array(g, data=[4, 0, 3]), axis=2))
    out["onehot"] = A(vk.U32Array(g, data=[0, 1, 2, 1, 0]).to_onehot(3))
    out["onehot2d"] = A(vk.U32Array(g, data=[[0, 1], [2, 1]]).to_onehot(3))
    return out


# ------------------------------------------------------------ random
@scenario()
def prng_streams(vk):
    g = vk.GPU()
    out = {}
    for size in (1, 3, 64, 100):
        r = vk.random.Xoshiro128pp(g, size=size, seed=12345)
        out[f"u32_{size}_a"] = A(r.randint(shape=(257,)))
        out[f"u32_{size}_b"] = A(r.randint(shape=(3, 5)))
        out[f"f32_{size}"] = A(r.random(shape=(130,)))
    r = vk.random.Xoshiro128pp(g, seed=0)
    out["seed0_5"] = A(r.random(shape=(5,)))
    out["seed0_65"] = A(r.random(shape=(65,)))
    r2 = vk.random.Xoshiro128pp(g, seed=2 ** 63 + 11)
    out["bigseed"] = A(r2.randint(shape=(70,)))
    r3 = vk.random.Xoshiro128pp(g, seed=7)
    out["range_3_4"] = A(r3.randrange(shape=(5,), low=3, high=4))
    out["range_10_1000"] = A(r3.randrange(shape=(200,), low=10, high=1000))
    out["range_big"] = A(r3.randrange(shape=(200,), low=5, high=2 ** 32))
    return out


@scenario(tol=("rtol", 1e-6, 4e-6))
def prng_normal_even(vk):
    g = vk.GPU()
    out = {}
    for size in (64, 4, 3):
        r = vk.random.Xoshiro128pp(g, size=size, seed=0)
        out[f"n{size}_10"] = A(r.normal(shape=(10,)))
        out[f"n{size}_ms"] = A(r.normal(shape=(6, 4), mean=5, stddev=3))
        out[f"n{size}_after"] = A(r.randint(shape=(9,))).astype(np.float32)
    return out


@scenario(tol=("rtol", 1e-6, 4e-6))
def prng_normal_odd(vk):
    # Odd n draws n+1 uniforms.  The reference dispatches n//2 pairs, but
    # whole 64-wide workgroups run, so the last element is written unless
    # (n//2) % 64 == 0 (then it stays unwritten: not exercised here).
    g = vk.GPU()
    out = {}
    for size in (64, 4, 3):
        r = vk.random.Xoshiro128pp(g, size=size, seed=0)
        out[f"n{size}_11"] = A(r.normal(shape=(11,)))
        out[f"n{size}_after"] = A(r.randint(shape=(9,))).astype(np.float32)
    r = vk.random.Xoshiro128pp(g, seed=0)
    out["doc_random3"] = A(r.random(shape=(3,)))
    out["doc_normal3"] = A(r.normal(shape=(3,)))
    return out


# ------------------------------------------------------------ nn
@scenario(tol=("rtol", 2e-6, 1e-6))
def nn_layers(vk):
    g = vk.GPU()
    nn = vk.nn
    out = {}
    relu = nn.ReLU()
    x = vk.Array(g, data=[[-0.2, 0.0, 0.2]])
    out["relu_y"] = A(relu(x))
    out["relu_dx"] = A(relu.backward(vk.Array(g, data=[[0.7, 0.8, 0.9]])))
    sig = nn.Sigmoid()
    d = np.asarray([[-100, -0.1, 0, 10, 100]])
    out["sig_y"] = A(sig(vk.Array(g, data=d)))
    out["sig_dx"] = A(sig.backward(vk.Array(g, data=[[0.1, 0.2, 0.3, 0.5, 0.7]])))
    sm = nn.Softmax()
    out["sm_y"] = A(sm(vk.Array(g, data=[[-10, -0.1, 0, 10, 12], [1.0, 1.0, 2.0, 0.5, -1.0]])))
    out["sm_dx"] = A(sm.backward(vk.Array(g, data=[[0.1, 0.2, 0.3, 0.5, 0.7], [1, 2, 3, 4, 5]])))
    dense = nn.Dense(g, 2, 2, w_init=nn.Constant(0.5), b_init=nn.Constant(1.0))
    out["dense_y"] = A(dense(vk.Array(g, data=[[1, 2], [3, 4]])))
    dense2 = nn.Dense(g, 2, 2, w_init=nn.Constant(0.25))
    dense2(vk.Array(g, data=[[1, 2], [3, 4]]))
    dx = dense2.backward(vk.Array(g, data=[[4, 2], [1, 3]]))
    out["dense_dW"] = A(dense2.w.grad); out["dense_db"] = A(dense2.b.grad); out["dense_dx"] = A(dx)
    return out


@scenario(tol=("rtol", 2e-6, 1e-7))
def nn_losses(vk):
    g = vk.GPU()
    nn = vk.nn
    out = {}
    _x = [[0.7, 0.3], [0.2, 0.8], [1.0, 0.0]]; _y = [[1.0, 0.0], [0.0, 1.0], [1.0, 0.0]]
    for red in ("mean", "sum"):
        ce = nn.CrossEntropyLoss(reduce=red)
        out[f"ce_{red}"] = A(ce(vk.Array(g, data=_x), vk.Array(g, data=_y)))
        out[f"ce_{red}_dx"] = A(ce.grad())
        sce = nn.SoftmaxCrossEntropyLoss(reduce=red)
        out[f"sce_{red}"] = A(sce(vk.Array(g, data=[[-1, 0], [10, 15]]), vk.Array(g, data=[[1, 0], [0, 1]])))
        out[f"sce_{red}_dx"] = A(sce.grad())
        mse = nn.MSELoss(reduce=red)
        out[f"mse_{red}"] = A(mse(vk.Array(g, data=[[4, 2], [1, 1.5]]), vk.Array(g, data=[[3, 2.2], [0.7, 1.5]])))
        out[f"mse_{red}_dx"] = A(mse.grad())
        hub = nn.HuberLoss(reduce=red)
        out[f"huber_{red}"] = A(hub(vk.Array(g, data=[[1.0, 2.2], [-3.0, 0.7]]),
                                    vk.Array(g, data=[[10, 3.0], [-5, 0.5]])))
        out[f"huber_{red}_dx"] = A(hub.grad())
    out["ce_equal"] = A(nn.CrossEntropyLoss()(vk.Array(g, data=[[0.5, 0.5]]), vk.Array(g, data=[[0.5, 0.5]])))
    return out


@scenario()
def nn_optimizers(vk):
    g = vk.GPU()
    nn = vk.nn
    out = {}
    grad = vk.Array(g, data=[1.0, -2.0, 3.0, 0.5])
    s = nn.SGD(lr=0.01).init_state(grad.shape)
    out["sgd"] = A(s.grad2diff(grad))
    adam = nn.Adam(g, lr=1e-3)
    st = adam.init_state(grad.shape)
    for i in range(3):
        out[f"adam_{i}"] = A(st.grad2diff(grad))
    ada = nn.AdaGrad(g, lr=0.05, tau=0.1)
    sa = ada.init_state(grad.shape)
    for i in range(3):
        out[f"adagrad_{i}"] = A(sa.grad2diff(grad))
    return out


@scenario(tol=("rtol", 1e-6, 1e-7))
def nn_regularizers(vk):
    g = vk.GPU()
    nn = vk.nn
    from_params = __import__(vk.__name__ + ".nn.parameters", fromlist=["Parameter"]).Parameter
    out = {}
    for v in (0.0, 3.5, -3.5):
        p = from_params(g, (2,), initializer=nn.Constant(v))
        for name, R in (("ridge", nn.Ridge(1.0)), ("lasso", nn.Lasso(0.5)), ("elastic", nn.Elastic(1.0, 2.0))):
            out[f"{name}_{v}_loss"] = A(R.loss(p.value))
            out[f"{name}_{v}_grad"] = A(R.grad(p.value))
    return out


@scenario(tol=("rtol", 5e-5, 5e-6))
def nn_train_steps(vk):
    """Sequence.train for a few steps: HeNormal init from fixed seeds (so the
    PRNG path is included), Adam, softmax cross entropy."""
    g = vk.GPU()
    nn = vk.nn
    rng = np.random.default_rng(3)
    X = rng.standard_normal((16, 12)).astype(np.float32)
    Y = np.eye(4, dtype=np.float32)[rng.integers(0, 4, 16)]
    opt = nn.Adam(g, lr=1e-2)
    net = nn.Sequence([
        nn.Dense(g, 12, 8, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(g, 12, seed=1)),
        nn.ReLU(),
        nn.Dense(g, 8, 8, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(g, 8, seed=2)),
        nn.Sigmoid(),
        nn.Dense(g, 8, 4, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(g, 8, seed=3)),
    ], nn.SoftmaxCrossEntropyLoss())
    out = {"w0_init": A(net.L[0].w.value).copy()}
    x = vk.Array(g, data=X); y = vk.Array(g, data=Y)
    for i in range(5):
        _y, loss = net.train(x, y)
        out[f"loss_{i}"] = A(loss).copy()
    out["pred"] = A(net.predict(x))
    out["w0"] = A(net.L[0].w.value); out["b2"] = A(net.L[4].b.value)
    return out


def backward_suite_inputs():
    """Seeded inputs of the layer / loss backward scenario (also used by the
    autograd tests, which compare their Functions with its golden values):
    logits and a gradient for the activations, probabilities and one-hot
    labels for cross entropy, predictions and targets for MSE / Huber with
    differences on both sides of the Huber kink (|d| = 1)."""
    rng = np.random.default_rng(17)
    z = rng.standard_normal((16, 7)).astype(np.float32) * np.float32(2)
    dy = rng.standard_normal((16, 7)).astype(np.float32)
    prob = rng.uniform(0.05, 1.0, (16, 7)).astype(np.float32)
    prob /= prob.sum(axis=1, keepdims=True)
    onehot = np.eye(7, dtype=np.float32)[rng.integers(0, 7, 16)]
    pred = rng.standard_normal((16, 7)).astype(np.float32)
    target = (pred + rng.standard_normal((16, 7)) * 1.5).astype(np.float32)
    return z, dy, prob, onehot, pred, target


@scenario(tol=("rtol", 2e-6, 1e-7))
def nn_backward_suite(vk):
    """Every layer's and loss's backward (and forward) on the seeded inputs
    above: ReLU, Sigmoid, Softmax (the reference's diagonal form), cross
    entropy, softmax cross entropy, MSE, Huber and a MixLoss of MSE and
    Huber, each with the mean reduction's 1/batch scaling."""
    g = vk.GPU()
    nn = vk.nn
    z, dy, prob, onehot, pred, target = backward_suite_inputs()
    out = {}
    for name, layer in (("relu", nn.ReLU()), ("sigmoid", nn.Sigmoid()), ("softmax", nn.Softmax())):
        out[f"{name}_y"] = A(layer(vk.Array(g, data=z)))
        out[f"{name}_dx"] = A(layer.backward(vk.Array(g, data=dy)))
    cases = (("ce", nn.CrossEntropyLoss(), prob, onehot), ("sce", nn.SoftmaxCrossEntropyLoss(), z, onehot),
             ("mse", nn.MSELoss(), pred, target), ("huber", nn.HuberLoss(), pred, target),
             ("mix", nn.losses.MixLoss([(0.3, nn.MSELoss()), (0.7, nn.HuberLoss())]), pred, target))
    for name, loss, x, y in cases:
        out[f"{name}_loss"] = A(loss(vk.Array(g, data=x), vk.Array(g, data=y)))
        out[f"{name}_dx"] = A(loss.grad())
    return out


# ------------------------------------------------------------ small op suite
def _suite_inputs():
    rng = np.random.default_rng(0)
    A_ = rng.uniform(-1, 1, size=(512, 1024)).astype(np.float32)
    B_ = rng.uniform(-1, 1, size=(1, 1024)).astype(np.float32)
    M1 = rng.standard_normal((256, 256)).astype(np.float32)
    M2 = rng.standard_normal((256, 256)).astype(np.float32)
    idx = rng.integers(0, 524288, 4096).astype(np.uint32)
    return A_, B_, M1, M2, idx


def _digest(x):
    """Rows 0-7 plus per-column float64 sums: small but covers every element."""
    x = np.asarray(x)
    if x.ndim == 2 and x.shape[0] > 8:
        return np.concatenate([x[:8].reshape(-1).astype(np.float64), x.astype(np.float64).sum(axis=0)])
    return x


@scenario(tol=("exact",))
def small_suite_exact(vk):
    g = vk.GPU()
    A_, B_, M1, M2, idx = _suite_inputs()
    a = vk.Array(g, data=A_); b = vk.Array(g, data=B_)
    out = {"add": _digest(a + b), "mul": _digest(a * b), "div_absp1": _digest(a / (b.abs() + 1.0)),
           "sq": _digest(a ** 2.0), "clamp": _digest(a.clamp(-0.5, 0.5)),
           "max0": A(a.maximum(axis=0)), "max1": A(a.maximum(axis=1)),
           "gather": A(a.gather(vk.U32Array(g, data=idx)))}
    return out


@scenario(tol=("ulp", 4))
def small_suite_math(vk):
    g = vk.GPU()
    A_, B_, M1, M2, idx = _suite_inputs()
    a = vk.Array(g, data=A_)
    return {"exp": A(a.exp())[:8], "tanh": A(a.tanh())[:8], "exp_rows": A(a.exp())[::61], "tanh_rows": A(a.tanh())[::61]}


@scenario(tol=("rtol", 2e-5, 2e-4))
def small_suite_reduce(vk):
    g = vk.GPU()
    A_, B_, M1, M2, idx = _suite_inputs()
    a = vk.Array(g, data=A_)
    return {"sum0": A(a.sum(axis=0)), "sum1": A(a.sum(axis=1)), "mean0": A(a.mean(axis=0)),
            "mean1": A(a.mean(axis=1))}


@scenario(tol=("rtol", 1e-4, 1e-4))
def small_suite_matmul(vk):
    g = vk.GPU()
    A_, B_, M1, M2, idx = _suite_inputs()
    return {"mm": _digest(vk.Array(g, data=M1) @ vk.Array(g, data=M2))}


@scenario()
def small_suite_prng(vk):
    g = vk.GPU()
    r = vk.random.Xoshiro128pp(g, size=64, seed=0)
    u = A(r.random(shape=(65536,)))
    return {"u_head": u[:1024], "u_sum": np.asarray([u.astype(np.float64).sum()]),
            "after": A(r.randint(shape=(256,)))}


@scenario(tol=("rtol", 1e-6, 4e-6))
def small_suite_normal(vk):
    g = vk.GPU()
    r = vk.random.Xoshiro128pp(g, size=64, seed=0)
    z = A(r.normal(shape=(65536,)))
    return {"z_head": z[:2048], "z_rows": z[::97]}
