"""Every golden scenario on the GB300 path against the reference's outputs
(tests/golden/golden.npz, produced by the reference's own Python)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import scenarios  # noqa: E402

from oracle.ops import ulp_distance  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "golden.npz"))

pytestmark = pytest.mark.gpu


def _compare(key, got, exp, tol):
    got = np.asarray(got)
    assert got.shape == exp.shape, f"{key}: shape {got.shape} vs {exp.shape}"
    kind = tol[0]
    if kind == "exact" or exp.dtype.kind in "ui":
        np.testing.assert_array_equal(got, exp, err_msg=key)
    elif kind == "ulp":
        d = ulp_distance(got.astype(np.float32), exp.astype(np.float64))
        finite = np.isfinite(exp)
        assert np.array_equal(np.isfinite(got), finite), key
        assert d[finite].max(initial=0) <= tol[1], f"{key}: {d[finite].max()} ulp > {tol[1]}"
    else:
        np.testing.assert_allclose(got, exp, rtol=tol[1], atol=tol[2], err_msg=key)


@pytest.mark.parametrize("name,fn,tol", scenarios.SCENARIOS, ids=[s[0] for s in scenarios.SCENARIOS])
def test_scenario_matches_reference(name, fn, tol):
    import vulkpy_gb300 as vk
    out = fn(vk)
    keys = [k for k in GOLDEN.files if k.startswith(name + "/")]
    assert len(keys) == len(out), f"{name}: {sorted(out)} vs {keys}"
    for k, v in out.items():
        _compare(f"{name}/{k}", v, GOLDEN[f"{name}/{k}"], tol)
