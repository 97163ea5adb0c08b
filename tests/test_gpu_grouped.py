"""Grouped GEMM and the grouped MLP training step.

* fp32 grouped products equal vkc_gemm's bit for bit (same tile code) except
  vector products (M == 1 or N == 1), which vkc_gemm runs as fp32 GEMV;
* split-bf16x3 grouped products equal vkc_gemm's bit for bit when that call
  does not split K (forced through the tuning table), and stay within the
  split method's 1e-5 relative error of float64;
* GroupedSequence.train leaves every model's parameters exactly where its
  own Sequence.train would, eagerly and replayed from a CUDA graph."""
import ctypes as C

import numpy as np
import pytest

from oracle.ops import rel_fro

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vk():
    import vulkpy_gb300
    return vulkpy_gb300


def _problems(rng, count):
    shapes = [(1, 1, 1), (1, 300, 7), (129, 257, 100), (17, 5, 1021), (300, 2, 64), (256, 1024, 784),
              (3, 2048, 33), (512, 64, 2048), (65, 129, 0), (0, 12, 9)]
    while len(shapes) < count:
        shapes.append((int(rng.integers(1, 513)), int(rng.integers(2, 2049)), int(rng.integers(1, 1100))))
    return shapes[:count]


def _run_grouped(vk, gpu, lib_, prec, specs):
    probs = []
    outs = []
    for (ta, tb, M, N, K, alpha, beta, A, B, C0, bias, act, mask) in specs:
        probs.append(lib_.GemmProblem(
            ta=ta, tb=tb, m=M, n=N, k=K, alpha=alpha, beta=beta, a=A._dptr() if K else None,
            lda=(M if ta else K), b=B._dptr() if K else None, ldb=(K if tb else N), c=C0._dptr(), ldc=N,
            bias=bias._dptr() if bias is not None else None, act=act,
            relu_mask=mask._dptr() if mask is not None else None))
        outs.append(C0)
    arr = (lib_.GemmProblem * len(probs))(*probs)
    st = lib_.lib.vkc_gemm_grouped(gpu.handle, prec, arr, len(probs))
    assert st == 0, lib_.last_error()
    for c in outs:
        c._written()
    return [np.asarray(c).copy() for c in outs]


def _specs(vk, gpu, rng, count, with_epilogue):
    specs, host = [], []
    for i, (M, N, K) in enumerate(_problems(rng, count)):
        ta, tb = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        A = rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32)
        B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
        C0 = rng.standard_normal((M, N)).astype(np.float32)
        alpha, beta = (1.0, 0.0) if not with_epilogue else (float(rng.choice([1.0, 0.5])), float(rng.choice([0.0, 2.0])))
        bias = rng.standard_normal(N).astype(np.float32) if with_epilogue and i % 2 else None
        act = int(rng.integers(0, 3)) if with_epilogue else 0
        mask = rng.standard_normal((M, N)).astype(np.float32) if with_epilogue and i % 3 == 0 else None
        host.append((ta, tb, M, N, K, alpha, beta, A, B, C0, bias, act, mask))
        specs.append((ta, tb, M, N, K, alpha, beta, vk.Array(gpu, data=A), vk.Array(gpu, data=B),
                      vk.Array(gpu, data=C0), None if bias is None else vk.Array(gpu, data=bias), act,
                      None if mask is None else vk.Array(gpu, data=mask)))
    return specs, host


def _expected(h):
    ta, tb, M, N, K, alpha, beta, A, B, C0, bias, act, mask = h
    opA = A.T if ta else A
    opB = B.T if tb else B
    v = alpha * (opA.astype(np.float64) @ opB.astype(np.float64)) + beta * C0
    if bias is not None:
        v = v + bias
    if act == 1:
        v = np.maximum(v, 0)
    elif act == 2:
        v = 1 / (1 + np.exp(-v))
    if mask is not None:
        v = v * (mask > 0)
    return v


def _single(vk, gpu, lib_, prec, spec):
    """The same problem through vkc_gemm (+ the separate ReLU-backward kernel
    for a mask) -- the per-op path the grouped call must reproduce."""
    ta, tb, M, N, K, alpha, beta, A, B, C0, bias, act, mask = spec
    assert bias is None and act == 0 and mask is None
    c = vk.Array(gpu, data=np.zeros((M, N), np.float32))
    st = lib_.lib.vkc_gemm(gpu.handle, prec, ta, tb, M, N, K, C.c_float(alpha), A._dptr() if K else None,
                           (M if ta else K), B._dptr() if K else None, (K if tb else N), C.c_float(beta), c._dptr(), N)
    assert st == 0, lib_.last_error()
    c._written()
    return np.asarray(c).copy()


@pytest.mark.parametrize("prec_name,bound", [("fp32", 2e-6), ("bf16x3", 1e-5), ("bf16", 8e-3)])
def test_grouped_accuracy_and_epilogue(gpu, vk, prec_name, bound):
    from vulkpy_gb300 import _lib as lib_
    prec = {"fp32": lib_.MM_FP32, "bf16": lib_.MM_BF16, "bf16x3": lib_.MM_BF16X3}[prec_name]
    rng = np.random.default_rng(11)
    specs, host = _specs(vk, gpu, rng, 24, with_epilogue=True)
    got = _run_grouped(vk, gpu, lib_, prec, specs)
    for g, h in zip(got, host):
        e = _expected(h)
        if e.size == 0:
            continue
        if not np.any(e):
            assert np.max(np.abs(g)) <= bound, (prec_name, h[2:5])
            continue
        assert rel_fro(g, e) < bound, (prec_name, h[2:5], rel_fro(g, e))
    assert gpu.check_errors() == 0


@pytest.mark.parametrize("prec_name", ["fp32", "bf16x3"])
def test_grouped_bit_identical_to_single(gpu, vk, prec_name):
    from vulkpy_gb300 import _lib as lib_, autotune
    prec = {"fp32": lib_.MM_FP32, "bf16x3": lib_.MM_BF16X3}[prec_name]
    rng = np.random.default_rng(5)
    specs, host = _specs(vk, gpu, rng, 20, with_epilogue=False)
    # the single-problem path must not split K for a bit-for-bit comparison
    for s in specs:
        assert lib_.lib.vkc_gemm_tune_set(lib_.MM_BF16X3, s[2], s[3], s[4], 1) == 0
        assert lib_.lib.vkc_gemm_tune_set(lib_.MM_FP32, s[2], s[3], s[4], 1) == 0
    try:
        fresh = [(ta, tb, M, N, K, a, b, A, B, vk.Array(gpu, data=np.zeros((M, N), np.float32)), bias, act, mask)
                 for (ta, tb, M, N, K, a, b, A, B, C0, bias, act, mask) in specs]
        got = _run_grouped(vk, gpu, lib_, prec, fresh)
        for g, s in zip(got, specs):
            M, N, K = s[2:5]
            if (M == 1 or N == 1) and K > 0:
                # vkc_gemm runs vector products as fp32 GEMV: the two agree to the
                # grouped call's precision
                assert rel_fro(g, _single(vk, gpu, lib_, prec, s)) < 2e-5, s[2:5]
                continue
            np.testing.assert_array_equal(g, _single(vk, gpu, lib_, prec, s), err_msg=str(s[2:5]))
    finally:
        lib_.lib.vkc_gemm_tune_clear()
        autotune.load_table()
    assert gpu.check_errors() == 0


def test_matmul_grouped_api(gpu, vk):
    rng = np.random.default_rng(2)
    As = [rng.standard_normal((m, k)).astype(np.float32) for m, k in [(3, 5), (64, 200), (130, 17)]]
    Bs = [rng.standard_normal((k, n)).astype(np.float32) for k, n in [(5, 9), (200, 1), (17, 300)]]
    for prec, bound in (("fp32", 1e-6), ("bf16x3", 1e-5)):
        outs = vk.vkarray.matmul_grouped([vk.Array(gpu, data=a) for a in As], [vk.Array(gpu, data=b) for b in Bs],
                                         precision=prec)
        for o, a, b in zip(outs, As, Bs):
            assert rel_fro(np.asarray(o), a.astype(np.float64) @ b) < bound
    with pytest.raises(ValueError):
        vk.vkarray.matmul_grouped([vk.Array(gpu, data=As[0])], [vk.Array(gpu, data=Bs[1])])


def _models(vk, gpu, dims, seed0=7):
    nn = vk.nn
    out = []
    for k, (i, h, o, b) in enumerate(dims):
        opt = nn.SGD(lr=1e-2)
        out.append(nn.Sequence([
            nn.Dense(gpu, i, h, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, i, seed=seed0 + k)), nn.ReLU(),
            nn.Dense(gpu, h, o, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, h, seed=seed0 + 1000 + k)),
        ], nn.MSELoss()))
    return out


def _params(models):
    return [np.asarray(p.value).copy() for m in models for d in (m.L[0], m.L[2]) for p in (d.w, d.b)]


@pytest.mark.parametrize("prec", ["fp32", "bf16x3"])
def test_grouped_sequence_matches_per_model_training(gpu, vk, prec):
    from vulkpy_gb300 import _lib as lib_, autotune
    rng = np.random.default_rng(2)
    dims = [(int(rng.integers(17, 1022)), int(rng.integers(32, 2049)), int(rng.integers(2, 65)),
             int(rng.integers(1, 513))) for _ in range(10)]
    data = [(rng.standard_normal((b, i)).astype(np.float32), rng.standard_normal((b, o)).astype(np.float32))
            for i, h, o, b in dims]
    xs = [vk.Array(gpu, data=x) for x, _ in data]
    ys = [vk.Array(gpu, data=y) for _, y in data]
    old = gpu.matmul_precision
    gpu.matmul_precision = prec
    # the per-model path must not split K (for bit-identity of the x3 sums)
    for (i, h, o, b) in dims:
        for (m, n, k) in ((b, h, i), (b, o, h), (o, h, b), (h, i, b), (b, h, o)):
            lib_.lib.vkc_gemm_tune_set(lib_.MM_BF16X3, m, n, k, 1)
            lib_.lib.vkc_gemm_tune_set(lib_.MM_FP32, m, n, k, 1)
    try:
        ref = _models(vk, gpu, dims)
        ref_losses = []
        for step in range(3):
            ref_losses.append([float(np.asarray(m.train(x, y)[1]).reshape(-1)[0]) for m, x, y in zip(ref, xs, ys)])
        grp_models = _models(vk, gpu, dims)
        grp = vk.nn.GroupedSequence(grp_models)
        grp_losses = []
        for step in range(3):
            preds, losses = grp.train(xs, ys)
            grp_losses.append(np.asarray(losses).tolist())
        for a, b in zip(_params(ref), _params(grp_models)):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_allclose(np.array(grp_losses), np.array(ref_losses), rtol=2e-6)

        # one captured step, replayed, continues exactly like eager steps
        g = vk.graph.Graph(gpu)
        with g:
            preds, losses = grp.train(xs, ys)
        for _ in range(2):
            g.launch()
            for m, x, y in zip(ref, xs, ys):
                m.train(x, y)
        for a, b in zip(_params(ref), _params(grp_models)):
            np.testing.assert_array_equal(a, b)
    finally:
        gpu.matmul_precision = old
        lib_.lib.vkc_gemm_tune_clear()
        autotune.load_table()
    assert gpu.check_errors() == 0


def test_grouped_sequence_rejects_unsupported(gpu, vk):
    nn = vk.nn
    sgd = nn.SGD(lr=0.1)
    a = nn.Sequence([nn.Dense(gpu, 3, 4, w_opt=sgd, b_opt=sgd), nn.ReLU(), nn.Dense(gpu, 4, 2, w_opt=sgd, b_opt=sgd)],
                    nn.MSELoss())
    b = nn.Sequence([nn.Dense(gpu, 3, 2, w_opt=sgd, b_opt=sgd)], nn.MSELoss())
    with pytest.raises(ValueError):
        nn.GroupedSequence([a, b])                       # different layer patterns
    with pytest.raises(NotImplementedError):
        nn.GroupedSequence([nn.Sequence([nn.Dense(gpu, 3, 2)], nn.CrossEntropyLoss())])
    with pytest.raises(NotImplementedError):
        nn.GroupedSequence([nn.Sequence([nn.Dense(gpu, 3, 2, w_opt=nn.Adam(gpu), b_opt=nn.Adam(gpu))],
                                        nn.MSELoss())])


def _update_pairs(vk, gpu, rng, shapes):
    """For each (batch, in, out): dy (batch x out), x (batch x in), W (out x in):
    dW = dy^T x with W's step fused, and dx = dy W, which reads W."""
    host, dev = [], []
    for b, i, o in shapes:
        dy = rng.standard_normal((b, o)).astype(np.float32)
        x = rng.standard_normal((b, i)).astype(np.float32)
        W = rng.standard_normal((o, i)).astype(np.float32)
        host.append((dy, x, W))
        dev.append(tuple(vk.Array(gpu, data=a) for a in (dy, x, W)) +
                   (vk.Array(gpu, shape=(o, i)), vk.Array(gpu, shape=(b, i))))
    return host, dev


def _pair_problems(lib_, shapes, dev):
    probs = []
    for (b, i, o), (dy, x, W, dW, dx) in zip(shapes, dev):
        probs.append(lib_.GemmProblem(ta=1, tb=0, m=o, n=i, k=b, alpha=1.0, beta=0.0, a=dy._dptr(), lda=o,
                                      b=x._dptr(), ldb=i, c=dW._dptr(), ldc=i, bias=None, act=0, relu_mask=None))
        probs.append(lib_.GemmProblem(ta=0, tb=0, m=b, n=i, k=o, alpha=1.0, beta=0.0, a=dy._dptr(), lda=o,
                                      b=W._dptr(), ldb=i, c=dx._dptr(), ldc=i, bias=None, act=0, relu_mask=None))
    return probs


@pytest.mark.parametrize("prec_name,pairs", [("fp32", 6), ("bf16", 6), ("bf16x3", 6), ("bf16x3", 70)])
def test_grouped_fused_update(gpu, vk, prec_name, pairs):
    """vkc_gemm_grouped_update: the gradients equal vkc_gemm_grouped's, dx
    reads W before its step, and W ends at W + float32(-lr) * dW in the SGD
    kernels' arithmetic -- in the epilogue (one launch) and through the
    separate update (fp32, K = 0, and 140 problems: more than one launch)."""
    from vulkpy_gb300 import _lib as lib_
    prec = {"fp32": lib_.MM_FP32, "bf16": lib_.MM_BF16, "bf16x3": lib_.MM_BF16X3}[prec_name]
    rng = np.random.default_rng(21)
    shapes = [(37, 300, 50), (256, 1024, 20), (200, 129, 130), (1, 17, 2), (0, 40, 8), (64, 65, 64)]
    while len(shapes) < pairs:
        shapes.append((int(rng.integers(1, 300)), int(rng.integers(2, 300)), int(rng.integers(2, 100))))
    shapes = shapes[:pairs]
    host, dev = _update_pairs(vk, gpu, rng, shapes)
    scale = np.float32(-0.01)
    # the same products without updates, on copies of W
    ref_dev = [(dy, x, vk.Array(gpu, data=h[2]), vk.Array(gpu, shape=dW.shape), vk.Array(gpu, shape=dx.shape))
               for (dy, x, W, dW, dx), h in zip(dev, host)]
    probs = _pair_problems(lib_, shapes, ref_dev)
    assert lib_.lib.vkc_gemm_grouped(gpu.handle, prec, (lib_.GemmProblem * len(probs))(*probs), len(probs)) == 0
    probs = _pair_problems(lib_, shapes, dev)
    upds = []
    for (dy, x, W, dW, dx) in dev:
        upds += [lib_.GemmUpdate(value=W._dptr(), scale=float(scale)), lib_.GemmUpdate(value=None, scale=0.0)]
    st = lib_.lib.vkc_gemm_grouped_update(gpu.handle, prec, (lib_.GemmProblem * len(probs))(*probs),
                                          (lib_.GemmUpdate * len(upds))(*upds), len(probs))
    assert st == 0, lib_.last_error()
    for (dy, x, W, dW, dx), (_, _, _, rdW, rdx), h in zip(dev, ref_dev, host):
        for a in (W, dW, dx, rdW, rdx):
            a._written()
        g = np.asarray(dW)
        np.testing.assert_array_equal(g, np.asarray(rdW))
        np.testing.assert_array_equal(np.asarray(dx), np.asarray(rdx))
        np.testing.assert_array_equal(np.asarray(W), h[2] + scale * g)
    assert gpu.check_errors() == 0


def test_grouped_fused_update_rejects(gpu, vk):
    from vulkpy_gb300 import _lib as lib_
    rng = np.random.default_rng(3)
    shapes = [(8, 16, 4)]
    _, dev = _update_pairs(vk, gpu, rng, shapes)
    dy, x, W, dW, dx = dev[0]
    bias = vk.Array(gpu, data=np.ones(16, np.float32))
    p = _pair_problems(lib_, shapes, dev)[0]
    for field, value in (("bias", bias._dptr()), ("alpha", 2.0), ("act", 1)):
        q = lib_.GemmProblem.from_buffer_copy(p)
        setattr(q, field, value)
        st = lib_.lib.vkc_gemm_grouped_update(gpu.handle, lib_.MM_BF16X3, C.byref(q),
                                              C.byref(lib_.GemmUpdate(value=W._dptr(), scale=-0.1)), 1)
        assert st != 0, field
    # the value may not be the problem's own C or operand
    st = lib_.lib.vkc_gemm_grouped_update(gpu.handle, lib_.MM_BF16X3, C.byref(p),
                                          C.byref(lib_.GemmUpdate(value=x._dptr(), scale=-0.1)), 1)
    assert st != 0


def test_colsum_update_grouped(gpu, vk):
    from vulkpy_gb300 import _lib as lib_
    rng = np.random.default_rng(4)
    shapes = [(5, 3), (256, 1024), (1, 40), (0, 7), (513, 65)]
    dys = [rng.standard_normal(s).astype(np.float32) for s in shapes]
    vals = [rng.standard_normal(s[1]).astype(np.float32) for s in shapes]
    scales = np.array([-0.01, -0.5, -1e-3, -0.25, -2.0], np.float32)
    d_dy = [vk.Array(gpu, data=d) if d.size else vk.Array(gpu, shape=d.shape) for d in dys]
    d_db = [vk.Array(gpu, shape=(s[1],)) for s in shapes]
    d_ref = [vk.Array(gpu, shape=(s[1],)) for s in shapes]
    d_val = [vk.Array(gpu, data=v) for v in vals]
    n = len(shapes)
    ptrs = lambda arrs: (C.c_void_p * n)(*[a._dptr() for a in arrs])
    rows = (C.c_int64 * n)(*[s[0] for s in shapes])
    cols = (C.c_int64 * n)(*[s[1] for s in shapes])
    assert lib_.lib.vkc_colsum_grouped(gpu.handle, ptrs(d_dy), ptrs(d_ref), rows, cols, n, 1) == 0
    st = lib_.lib.vkc_colsum_update_grouped(gpu.handle, ptrs(d_dy), ptrs(d_db), rows, cols, n, 1, ptrs(d_val),
                                            (C.c_float * n)(*scales))
    assert st == 0, lib_.last_error()
    for db, ref, v, v0, s in zip(d_db, d_ref, d_val, vals, scales):
        for a in (db, ref, v):
            a._written()
        g = np.asarray(db)
        np.testing.assert_array_equal(g, np.asarray(ref))
        np.testing.assert_array_equal(np.asarray(v), v0 + s * g)
    assert gpu.check_errors() == 0
