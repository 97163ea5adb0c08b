"""Generate tests/golden/golden.npz by running every scenario in scenarios.py
on the reference's own Python package over the oracle's fake native module.

Run where the reference source tree exists:
    python tests/golden/make_golden.py [--reference /path/to/reference]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def run_reference(reference_root: str) -> dict:
    from oracle.fake_vkarray import load_reference
    import scenarios
    vk = load_reference(reference_root)
    out = {}
    for name, fn, tol in scenarios.SCENARIOS:
        res = fn(vk)
        for k, v in res.items():
            out[f"{name}/{k}"] = np.asarray(v)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("VULKPY_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")))
    ap.add_argument("--out", default=os.path.join(HERE, "golden.npz"))
    args = ap.parse_args()
    out = run_reference(args.reference)
    np.savez_compressed(args.out, **out)
    print(f"wrote {len(out)} arrays to {args.out} ({os.path.getsize(args.out)} bytes)")


if __name__ == "__main__":
    main()
