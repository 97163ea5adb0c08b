"""Host-side logic that needs no GPU: axis normalisation of the reductions and
the autotuner's table merge when one precision is re-tuned."""
import json
import sys

import numpy as np
import pytest


def test_normalize_axes_matches_numpy_semantics():
    from vulkpy_gb300.vkarray import _normalize_axes
    assert _normalize_axes(0, 2) == [0]
    assert _normalize_axes(-1, 3) == [2]
    assert _normalize_axes((0, 2), 3) == [2, 0]
    assert _normalize_axes([1, -2, 1], 3) == [1]          # duplicates collapse, descending order
    assert _normalize_axes(np.int64(1), 2) == [1]
    assert _normalize_axes(np.array([0, 2]), 3) == [2, 0]
    assert _normalize_axes((np.int32(0), 1), 2) == [1, 0]
    for bad in (2, -3, (0, 3)):
        with pytest.raises(ValueError):
            _normalize_axes(bad, 2)


def test_autotune_only_keeps_other_precisions(tmp_path, monkeypatch):
    """`--only fp32` writes the new fp32 entries and the existing bf16x3/bf16
    entries unchanged (tune() itself needs a GPU and is replaced here)."""
    from vulkpy_gb300 import autotune
    old = {"bf16x3": [[8, 10, 10, 2, 128]], "bf16": [[8, 10, 10, 3, 256]], "fp32": [[8, 8, 8, 4, 256]]}
    table_path = tmp_path / "tuning.json"
    table_path.write_text(json.dumps(old))
    out = tmp_path / "new.json"
    calls = {}

    def fake_tune(shapes=None, verbose=True, only=None):
        calls["only"] = only
        return {"fp32": [[8, 8, 8, 16, 256]], "device": "test", "when": "now", "candidates": [1],
                "tiles": [256], "entry": "[log2 M, log2 N, log2 K, splits, tile width]"}

    monkeypatch.setattr(autotune, "tune", fake_tune)
    monkeypatch.setattr(autotune, "TABLE_PATH", str(table_path))
    monkeypatch.setattr(sys, "argv", ["autotune", "--only", "fp32", "--out", str(out)])
    autotune.main()
    new = json.loads(out.read_text())
    assert calls["only"] == "fp32"
    assert new["fp32"] == [[8, 8, 8, 16, 256]]
    assert new["bf16x3"] == old["bf16x3"] and new["bf16"] == old["bf16"]
