"""The differentiable-MLP workload (Dense 784-1024-ReLU-1024-Sigmoid-10,
softmax cross entropy, Adam 1e-3, HeNormal seed 1, one batch of 256) trained
for 1000 steps on this package against the loss curve the reference's own
Python computes for it (tests/golden/c4_loss_curve.npz, made by tests/golden/make_c4_curve.py
over the oracle's fake native module)."""
import importlib.util
import os

import numpy as np
import pytest

from oracle.ops import rel_fro

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "c4_loss_curve.npz")


def _build():
    spec = importlib.util.spec_from_file_location("_c4", os.path.join(HERE, "golden", "make_c4_curve.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build


# measured over the 1000 steps: fp32 2.4e-6 / 1.4e-5, split-bf16x3 4.0e-7 / 7.8e-6
# (loss deviation / last-layer weights)
@pytest.mark.parametrize("prec,loss_tol,w_tol", [("fp32", 2e-5, 1e-4), ("bf16x3", 2e-5, 1e-4)])
def test_loss_curve_matches_reference(gpu, prec, loss_tol, w_tol):
    import vulkpy_gb300 as vk
    if not os.path.exists(FIXTURE):
        pytest.skip("tests/golden/c4_loss_curve.npz not generated (tests/golden/make_c4_curve.py)")
    ref = np.load(FIXTURE)
    steps = int(ref["steps"][0])
    net, x, y = _build()(vk)
    g = x._gpu                       # the workload opens its own GPU object
    old = g.matmul_precision
    g.matmul_precision = prec
    try:
        losses = np.empty(steps, np.float32)
        for i in range(steps):
            _, loss = net.train(x, y)
            losses[i] = np.asarray(loss).reshape(-1)[0]
        w_last = np.asarray(net.L[4].w.value).copy()
    finally:
        g.matmul_precision = old
    # the first step's loss depends only on the initial weights and the data
    np.testing.assert_allclose(losses[0], ref["loss"][0], rtol=1e-5)
    # then float32 summation orders differ (reference: serial sums; here: tiled
    # GEMMs), and the curves stay within loss_tol (relative to the initial loss)
    dev = np.abs(losses - ref["loss"]) / ref["loss"][0]
    assert dev.max() <= loss_tol, (dev.max(), int(dev.argmax()))
    assert losses[-1] < 0.5 * losses[0]          # it trains
    assert rel_fro(w_last, ref["w_last"]) < w_tol
