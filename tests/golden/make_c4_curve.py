"""Generate tests/golden/c4_loss_curve.npz: the training-loss curve of the
differentiable-MLP workload as the reference computes it.

Workload (numpy seed 1 for the data, HeNormal seed 1 for every layer):
Dense 784->1024, ReLU, Dense 1024->1024, Sigmoid, Dense 1024->10,
SoftmaxCrossEntropyLoss, Adam(lr 1e-3, betas 0.9/0.999, eps 1e-8),
Ridge(1e-4) on every parameter (which vulkpy's Sequence never applies,
nn/models.py:55-78), one fixed batch of 256 N(0,1) rows with one-hot labels
from integers(0, 10, 256); `steps` training steps.

The reference's own Python (vulkpy/nn, vkarray.py, random.py) runs over the
oracle's fake native module, about 12 s per step on 8 cores (its Dense
backward materialises a 256 x 1024 x 1024 array), so 1000 steps take a few
hours; the file is rewritten every --save-every steps with the steps done
so far (and the last layer's weights after them), so an interrupted run
still leaves a consistent, shorter curve.  Run where the reference source
tree exists:
    python tests/golden/make_c4_curve.py [--steps 1000] [--reference PATH]
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def build(vk):
    """The workload on any module with vulkpy's API: (net, x, y)."""
    nn = vk.nn
    g = vk.GPU()
    rng = np.random.default_rng(1)
    X = rng.standard_normal((256, 784)).astype(np.float32)
    Y = np.eye(10, dtype=np.float32)[rng.integers(0, 10, 256)]
    opt = nn.Adam(g, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8)
    R = nn.Ridge(1e-4)
    net = nn.Sequence([
        nn.Dense(g, 784, 1024, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(g, 784, seed=1), w_reg=R, b_reg=R),
        nn.ReLU(),
        nn.Dense(g, 1024, 1024, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(g, 1024, seed=1), w_reg=R, b_reg=R),
        nn.Sigmoid(),
        nn.Dense(g, 1024, 10, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(g, 1024, seed=1), w_reg=R, b_reg=R),
    ], nn.SoftmaxCrossEntropyLoss())
    return net, vk.Array(g, data=X), vk.Array(g, data=Y)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("VULKPY_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")))
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--save-every", type=int, default=100)
    ap.add_argument("--out", default=os.path.join(HERE, "c4_loss_curve.npz"))
    args = ap.parse_args()
    from oracle.fake_vkarray import load_reference
    vk = load_reference(args.reference)
    net, x, y = build(vk)
    losses = np.empty(args.steps, dtype=np.float32)
    t0 = time.time()

    def save(done):
        tmp = args.out + ".tmp.npz"
        np.savez_compressed(tmp, loss=losses[:done], steps=np.array([done]),
                            w_last=np.asarray(net.L[4].w.value).copy(), b_last=np.asarray(net.L[4].b.value).copy())
        os.replace(tmp, args.out)
        print(f"wrote {args.out} ({done} steps)", flush=True)

    for i in range(args.steps):
        _, loss = net.train(x, y)
        losses[i] = np.asarray(loss).reshape(-1)[0]
        if i % 50 == 0:
            print(f"step {i}: loss {losses[i]:.6f} ({time.time() - t0:.0f} s)", flush=True)
        if (i + 1) % args.save_every == 0 and i + 1 < args.steps:
            save(i + 1)
    save(args.steps)


if __name__ == "__main__":
    main()
