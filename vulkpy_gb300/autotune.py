"""
Autotuner for the GEMMs: CTA tile width and split-K count of the tensor-core
GEMM (bf16 and split-bf16x3), split-K count of the fp32 SIMT GEMM.

For each size bucket (ceil(log2) of M, N and K) the tuner times every
candidate (tile width 256 or 128, split count) on a representative problem of
that bucket and keeps the fastest.  The result is written to ``tuning.json`` next to this file and
loaded into the library at import (vkc_gemm_tune_set), so the choice at run
time is a table lookup: deterministic, the same in eager runs and graph
captures.  Buckets without an entry fall back to an occupancy heuristic.

Run on the GPU:
    python -c "import vulkpy_gb300.autotune as t; t.main()" [--quick] [--only fp32] [--out FILE]
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import time
from typing import Dict, Iterable, List, Tuple

import numpy as np

from . import _lib
from ._lib import lib, check

TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")
CANDIDATES = (1, 2, 3, 4, 6, 8, 12, 16)   # split-K counts
TILES = (256, 128)                         # CTA tile widths (columns of C)


def bucket(x: int) -> int:
    b = 0
    while (1 << b) < x:
        b += 1
    return b


def load_table(path: str = TABLE_PATH) -> int:
    """Load the tuning table into the library; returns the entry count."""
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        data = json.load(f)
    n = 0
    for name, prec in (("bf16x3", _lib.MM_BF16X3), ("bf16", _lib.MM_BF16), ("fp32", _lib.MM_FP32)):
        for entry in data.get(name, []):
            m, nn, k, splits = entry[:4]
            tile = int(entry[4]) if len(entry) > 4 else 256
            # representative sizes: the top of each bucket
            check(lib.vkc_gemm_plan_set(prec, 1 << m, 1 << nn, 1 << k, int(splits), tile))
            n += 1
    return n


def default_shapes() -> List[Tuple[int, int, int]]:
    """Shapes of the MLP workloads (batch 256, 784-1024-1024-10 forward and
    backward), the batched uneven MLPs, and square / skinny sizes."""
    shapes = set()
    for (i, o) in ((784, 1024), (1024, 1024), (1024, 10)):
        for b in (256,):
            shapes.add((b, o, i))      # forward  x W^T
            shapes.add((o, i, b))      # dW = dy^T x
            shapes.add((b, i, o))      # dx = dy W
    rng = np.random.default_rng(2)
    for _ in range(64):
        i_ = int(rng.integers(17, 1022)); h_ = int(rng.integers(32, 2049))
        o_ = int(rng.integers(2, 65)); b_ = int(rng.integers(1, 513))
        for s in ((b_, h_, i_), (b_, o_, h_), (h_, i_, b_), (o_, h_, b_), (b_, h_, o_)):
            shapes.add(s)
    for s in (256, 512, 1024, 2048, 4096):
        shapes.add((s, s, s))
        shapes.add((128, s, 4 * s))
    # one representative per bucket
    rep: Dict[Tuple[int, int, int], Tuple[int, int, int]] = {}
    for (m, n, k) in sorted(shapes):
        rep.setdefault((bucket(m), bucket(n), bucket(k)), (m, n, k))
    return sorted(rep.values())


def _time_gemm(gpu, a, b, c, m, n, k, reps=5, calls=16, prec=None) -> float:
    """Device time of one call in ms.  The calls are captured in a CUDA
    graph and replayed, so host-side launch cost (which a graph removes)
    does not decide the choice."""
    lib_ = lib
    h = gpu.handle
    prec = _lib.MM_BF16X3 if prec is None else prec

    def run():
        check(lib_.vkc_gemm(h, prec, 0, 1, m, n, k, C.c_float(1.0), a, k, b, k, C.c_float(0.0), c, n))

    run()
    check(lib_.vkc_device_synchronize(h))
    check(lib_.vkc_graph_begin(h))
    try:
        for _ in range(calls):
            run()
    finally:
        g = C.c_void_p()
        st = lib_.vkc_graph_end(h, C.byref(g))
    check(st)
    try:
        check(lib_.vkc_graph_launch(g))
        times = []
        for _ in range(reps):
            t0, t1 = C.c_void_p(), C.c_void_p()
            check(lib_.vkc_timer_record(h, C.byref(t0)))
            check(lib_.vkc_graph_launch(g))
            check(lib_.vkc_timer_record(h, C.byref(t1)))
            ms = C.c_float()
            check(lib_.vkc_job_elapsed_ms(t0, t1, C.byref(ms)))
            lib_.vkc_job_destroy(t0)
            lib_.vkc_job_destroy(t1)
            times.append(ms.value / calls)
    finally:
        check(lib_.vkc_device_synchronize(h))
        lib_.vkc_graph_destroy(g)
    return float(np.median(times))


def tune(shapes: Iterable[Tuple[int, int, int]] = None, verbose: bool = True, only: str = None) -> dict:
    import vulkpy_gb300 as vk
    gpu = vk.GPU()
    shapes = list(shapes or default_shapes())
    check(lib.vkc_gemm_tune_clear())
    table = {}
    for name, prec in (("bf16x3", _lib.MM_BF16X3), ("bf16", _lib.MM_BF16), ("fp32", _lib.MM_FP32)):
        if only is not None and name != only:
            continue
        entries = []
        tiles = TILES if prec != _lib.MM_FP32 else (256,)   # the SIMT GEMM has one tile shape
        for (m, n, k) in shapes:
            rng = np.random.default_rng(m * 31 + n * 7 + k)
            A = vk.Array(gpu, data=rng.standard_normal((m, k)).astype(np.float32))
            B = vk.Array(gpu, data=rng.standard_normal((n, k)).astype(np.float32))
            Cm = vk.Array(gpu, shape=(m, n))
            nk = (k + 15) // 16 if prec == _lib.MM_FP32 else (k + 63) // 64   # K steps / K blocks
            best, best_ms = (1, 256), float("inf")
            results = {}
            for tile in tiles:
                for s in CANDIDATES:
                    if s > max(1, nk):
                        continue
                    check(lib.vkc_gemm_plan_set(prec, m, n, k, s, tile))
                    ms = _time_gemm(gpu, A._dptr(), B._dptr(), Cm._buf.ptr, m, n, k, prec=prec)
                    results[f"{tile}/{s}"] = round(ms * 1e3, 1)
                    if ms < best_ms:
                        best, best_ms = (s, tile), ms
            check(lib.vkc_gemm_plan_set(prec, m, n, k, best[0], best[1]))
            entries.append([bucket(m), bucket(n), bucket(k), best[0], best[1]])
            if verbose:
                print(f"{name} M={m} N={n} K={k}: best tile {best[1]} splits {best[0]} "
                      f"({best_ms * 1e3:.1f} us)  {results}", flush=True)
        table[name] = entries
    table.update({"device": vk.GPU()._dev.name, "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
                  "candidates": list(CANDIDATES), "tiles": list(TILES),
                  "entry": "[log2 M, log2 N, log2 K, splits, tile width]"})
    return table


def main():
    """``--only NAME`` re-tunes one precision (bf16x3, bf16 or fp32) and keeps
    the other precisions' entries of the existing table."""
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    table = tune(default_shapes()[:12] if "--quick" in sys.argv else None, only=only)
    out = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else TABLE_PATH
    if only is not None and os.path.exists(TABLE_PATH):
        with open(TABLE_PATH) as f:
            old = json.load(f)
        for name in ("bf16x3", "bf16", "fp32"):
            if name != only:
                table[name] = old.get(name, [])
    with open(out, "w") as f:
        json.dump(table, f, indent=1)
    print(f"wrote {sum(len(table[k]) for k in ('bf16x3', 'bf16', 'fp32'))} entries to {out}")


if __name__ == "__main__":
    main()
