"""
Benchmark: the bandwidth-bound float32 suite on one (or N replica) GB300.

Workload (seed 0, numpy default_rng, drawn in this order):
  X   = standard_normal (8192, 32768) float32          (1 GiB, larger than L2)
  row = uniform[0.5, 2) (1, 32768);  col = uniform[0.5, 2) (8192, 1)
  idx = integers(0, 2^28, 2^26) uint32
  Xoshiro128pp(size=2^20, seed=0)
One step, in order (all through the vulkpy API):
  X op row, X op col for op in + - * / ** max min          14 launches, 8 B/el
  Z = |X| + 1e-3; sqrt(Z), invsqrt(Z), log(Z), Z.sqrt(inplace)  6 launches, 8 B/el
  E = exp(X * 1e-4)                                          2 launches, 8 B/el
  sum, maximum, minimum, mean of X and prod of E over
    axis 0, axis 1, None                                    15 reductions, 4 B/el
  X.gather(idx)                                              12 B/index
  rng.random / normal / randint into 2^28-element buffers    4 B/out + 32 B/state
  X op= row, X op= col for op in + - * /  (in place)         8 launches, 8 B/el
metric = algorithmic bytes of the step / step time (GB/s).  Inputs stay in
HBM for `value`; the `e2e` leg uploads X, row, col, idx from pinned host
memory and reads the reduction results and the final X back every step
(pipelined: step i's read-back and step i+1's upload overlap the compute;
20 steps per timed repetition, best of eight repetitions).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ROWS, COLS = 8192, 32768
N_IDX = 1 << 26
PRNG_STATES = 1 << 20
METRIC = "ew HBM GB/s (bandwidth suite, fp32 8192x32768)"
BIN_OPS = ["__add__", "__sub__", "__mul__", "__truediv__", "__pow__", "max", "min"]
INPLACE_OPS = ["__iadd__", "__isub__", "__imul__", "__itruediv__"]


def step_bytes(rows, cols, n_idx, states):
    n = rows * cols
    b = 0
    b += 14 * (8 * n) + 7 * 4 * cols + 7 * 4 * rows      # broadcast binary
    b += 6 * 8 * n                                       # abs, +1e-3, 3 unary, in-place sqrt
    b += 2 * 8 * n                                       # E = exp(X * 1e-4)
    b += 15 * 4 * n + 5 * 4 * (cols + rows + 1)          # reductions (+ outputs)
    b += 12 * n_idx                                      # gather
    b += 3 * (4 * n + 32 * states)                       # PRNG random / normal / randint
    b += 8 * (8 * n) + 4 * 4 * cols + 4 * 4 * rows       # in-place broadcast
    return b


def bcast_bytes(rows, cols):
    return 8 * rows * cols + 4 * max(rows, cols)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_index: str):
        self.rows = []
        self.proc = None
        self.gpu_index = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", self.gpu_index], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = sorted({self.REASONS[i] for r in self.rows for i in range(4) if "Active" == r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------- GPU suite
class Timer:
    def __init__(self, vk, gpu):
        from vulkpy_gb300 import _lib
        import ctypes
        self.C, self.lib, self.h = ctypes, _lib.lib, gpu.handle

    def mark(self):
        j = self.C.c_void_p()
        assert self.lib.vkc_timer_record(self.h, self.C.byref(j)) == 0
        return j

    def ms(self, a, b):
        out = self.C.c_float()
        assert self.lib.vkc_job_elapsed_ms(a, b, self.C.byref(out)) == 0
        return out.value

    def free(self, *js):
        for j in js:
            self.lib.vkc_job_destroy(j)


def run_step(vk, X, row, col, idx, rng, U, Nrm, I, timer=None, spans=None, keep=None):
    """One step of the suite.  With `timer`, each broadcast-binary launch is
    bracketed by timing markers appended to `spans`."""
    for other in (row, col):
        for op in BIN_OPS:
            if timer is not None:
                a = timer.mark()
            r = getattr(X, op)(other)
            if timer is not None:
                spans.append((a, timer.mark()))
            del r
    Z = X.abs()
    Z += 1e-3
    for name in ("sqrt", "invsqrt", "log"):
        t = getattr(Z, name)()
        del t
    Z.sqrt(inplace=True)
    E = X * 1e-4
    E.exp(inplace=True)
    outs = []
    for axis in (0, 1, None):
        outs.append(X.sum(axis=axis))
        outs.append(X.maximum(axis=axis))
        outs.append(X.minimum(axis=axis))
        outs.append(X.mean(axis=axis))
        outs.append(E.prod(axis=axis))
    g = X.gather(idx)
    rng.random(buffer=U)
    rng.normal(buffer=Nrm)
    rng.randint(buffer=I)
    for other in (row, col):
        for op in INPLACE_OPS:
            getattr(X, op)(other)
    if keep is not None:
        keep.extend(outs)
    return outs, g


def make_inputs(rows, cols, n_idx):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((rows, cols), dtype=np.float32)
    row = rng.uniform(0.5, 2.0, (1, cols)).astype(np.float32)
    col = rng.uniform(0.5, 2.0, (rows, 1)).astype(np.float32)
    idx = rng.integers(0, rows * cols, n_idx, dtype=np.uint32)
    return X, row, col, idx


def max_over_ranks(x: float, dist) -> float:
    """The largest value of `x` over all ranks (the slowest rank's time);
    `x` itself without a process group."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def gpu_arm(args, rank, world, dist):
    import vulkpy_gb300 as vk
    from vulkpy_gb300 import _lib
    import ctypes

    local = int(os.environ.get("LOCAL_RANK", "0"))
    gpu = vk.GPU(local)
    rows, cols, n_idx, states = args.rows, args.cols, args.n_idx, args.states
    Xh, rowh, colh, idxh = make_inputs(rows, cols, n_idx)
    X = vk.Array(gpu, data=Xh)
    row, col = vk.Array(gpu, data=rowh), vk.Array(gpu, data=colh)
    idx = vk.U32Array(gpu, data=idxh)
    rng = vk.random.Xoshiro128pp(gpu, size=states, seed=0)
    n = rows * cols
    U, Nrm, I = vk.Array(gpu, shape=(n,)), vk.Array(gpu, shape=(n,)), vk.U32Array(gpu, shape=(n,))
    timer = Timer(vk, gpu)
    nbytes = step_bytes(rows, cols, n_idx, states)

    for _ in range(args.warmup):
        run_step(vk, X, row, col, idx, rng, U, Nrm, I)
    gpu.wait()

    clocks = ClockSampler(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0])
    clocks.start()
    time.sleep(0.3)
    spans = []
    lc0 = ctypes.c_uint64()
    _lib.lib.vkc_launch_count(ctypes.byref(lc0))
    if dist is not None:
        dist.barrier()
    gpu.wait()
    t0 = timer.mark()
    for _ in range(args.steps):
        run_step(vk, X, row, col, idx, rng, U, Nrm, I, timer=timer, spans=spans)
    t1 = timer.mark()
    gpu.wait()
    lc1 = ctypes.c_uint64()
    _lib.lib.vkc_launch_count(ctypes.byref(lc1))
    ms_total = timer.ms(t0, t1)
    clk = clocks.stop()
    bc_ms = [timer.ms(a, b) for a, b in spans]
    timer.free(t0, t1, *[j for s in spans for j in s])
    ms_total = max_over_ranks(ms_total, dist)
    ms_step = ms_total / args.steps
    value = world * nbytes / (ms_step * 1e-3) / 1e9
    launches = int(lc1.value - lc0.value)

    # roofline of the dominant kernel: the broadcast-binary launches
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = json.load(open(peaks_path))["hbm_gbs"]
        peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    else:
        peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    avg_bc = float(np.mean(bc_ms))
    achieved = bcast_bytes(rows, cols) / (avg_bc * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get("broadcast_binary_bytes_per_launch")
    roofline = {"kernel": "k_bcast_rows (X op row / X op col)", "bound": "hbm", "achieved": round(achieved, 1),
                "peak": peak, "peak_source": peak_src, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic, "algorithmic_bytes": bcast_bytes(rows, cols), "avg_ms": round(avg_bc, 4),
                "launches_timed": len(bc_ms)}

    # per-op breakdown from one extra, separately timed step (not in `value`)
    breakdown = profile_ops(vk, gpu, timer, X, row, col, idx, rng, U, Nrm, I)

    e2e = e2e_leg(vk, gpu, args, Xh, rowh, colh, idxh, rng, U, Nrm, I, nbytes, world, dist)
    del X, U, Nrm, I, idx
    extra = {}
    if not args.no_extra:
        extra["matmul"] = matmul_study(vk, gpu, timer)
        extra["mlp"] = mlp_study(vk, gpu, timer)
        extra["batched"] = batched_study(vk, gpu, timer)
        extra["chain"] = chain_study(vk, gpu, timer)
        extra["reduction_precision"] = reduction_precision_study(vk, gpu, timer)
        extra["train_loop"] = train_loop_study(vk, gpu)
        extra["small_suite"] = small_suite_study(vk, gpu, timer)

    result = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (numpy default_rng seed 0)",
        "config": {"workload": f"bandwidth suite: X ({rows},{cols}) fp32 N(0,1), row (1,{cols}), col ({rows},1) "
                               f"U[0.5,2); 49 ops/step (see bench.py docstring)",
                   "rows": rows, "cols": cols, "gather_indices": n_idx, "prng_states": states,
                   "bytes_per_step": nbytes, "l2": "inputs larger than L2 (1 GiB per array), no flush",
                   "parallelism": f"replicas x{world}"},
        "roofline": roofline, "e2e": e2e, "clocks": clk, "gpu_launches": launches, "ops_gbs": breakdown,
    }
    result.update(extra)
    return result


def profile_ops(vk, gpu, timer, X, row, col, idx, rng, U, Nrm, I):
    rows, cols = X.shape
    n = rows * cols
    fams = {}

    def timed(name, nbytes, fn, reps=4):
        # `reps` calls back to back: the host queues the later calls while
        # the first runs, so only one call's launch latency is in the span
        a = timer.mark()
        for _ in range(reps):
            r = fn()
        b = timer.mark()
        gpu.wait()
        ms = timer.ms(a, b) / reps
        timer.free(a, b)
        fams.setdefault(name, []).append(nbytes / (ms * 1e-3) / 1e9)
        return r

    gpu.wait()
    timed("bcast_row", 8 * n, lambda: X + row)
    timed("bcast_col", 8 * n, lambda: X * col)
    Z = timed("unary_abs", 8 * n, lambda: X.abs())
    Z += 1e-3  # log on |X| + 1e-3, as in the step
    timed("unary_log", 8 * n, lambda: Z.log())
    timed("scalar_mul", 8 * n, lambda: X * 1e-4)
    timed("sum_axis0", 4 * n, lambda: X.sum(axis=0))
    timed("sum_axis1", 4 * n, lambda: X.sum(axis=1))
    timed("sum_all", 4 * n, lambda: X.sum())
    timed("max_all", 4 * n, lambda: X.maximum())
    timed("gather_12B", 12 * idx.size, lambda: X.gather(idx))
    timed("prng_f32", 4 * n + 32 * rng.size, lambda: rng.random(buffer=U))
    timed("prng_normal", 4 * n + 32 * rng.size, lambda: rng.normal(buffer=Nrm))
    timed("prng_u32", 4 * n + 32 * rng.size, lambda: rng.randint(buffer=I))
    timed("inplace_bcast", 8 * n, lambda: X.__iadd__(row), reps=1)
    X -= row
    return {k: round(float(np.median(v)), 1) for k, v in fams.items()}


def e2e_leg(vk, gpu, args, Xh, rowh, colh, idxh, rng, U, Nrm, I, nbytes, world, dist):
    """Same step through the public API from pinned host buffers: uploads of
    X, row, col, idx and read-back of the reductions and the final X are
    inside the timed region, every step.  Pipelined as a user would write
    it: step i's results start copying back (``prefetch``) as soon as its ops
    are issued, step i+1's uploads and ops are issued next, and only then
    does the host read step i's results -- so step i's read-back and step
    i+1's upload overlap the compute instead of adding to it."""
    pins = []
    for h in (Xh, rowh, colh, idxh):
        p_ = vk.vkarray.empty_pinned(h.shape, h.dtype)
        p_[...] = h
        pins.append(p_)
    Xp, rowp, colp, idxp = pins
    h2d = sum(p_.nbytes for p_ in pins)
    d2h = 0

    def issue():
        X = vk.Array(gpu, data=Xp)
        row, col = vk.Array(gpu, data=rowp), vk.Array(gpu, data=colp)
        idx = vk.U32Array(gpu, data=idxp)
        outs, g = run_step(vk, X, row, col, idx, rng, U, Nrm, I)
        for o in outs:
            o.prefetch()
        X.prefetch()
        return outs, X

    def collect(pending):
        nonlocal d2h
        outs, X = pending
        got = [np.asarray(o) for o in outs]
        final = np.asarray(X)
        d2h = sum(o.nbytes for o in got) + final.nbytes

    import ctypes
    import gc
    from vulkpy_gb300 import _lib
    marks = []
    misses = []   # per iteration: (pinned host blocks, device allocations requested, issue ms,
                  #                 MiB the compute / upload pools grew by)
    gcs = []      # garbage collections (generation, ms) during the timed iterations

    def on_gc(phase, info):
        if phase == "start":
            on_gc.t = time.perf_counter()
        else:
            gcs.append((len(marks), info.get("generation"), round((time.perf_counter() - on_gc.t) * 1e3, 2)))
    on_gc.t = 0.0

    def counts():
        c, rc, ru = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _lib.lib.vkc_alloc_count(ctypes.byref(c))
        _lib.lib.vkc_pool_reserved(gpu.handle, ctypes.byref(rc), ctypes.byref(ru))
        return vk.vkarray._pinned_pool.allocs, c.value, rc.value, ru.value

    def run(steps):
        pending = None
        for _ in range(steps):
            c0 = counts()
            ta = time.perf_counter()
            cur = issue()
            tb = time.perf_counter()
            if pending is not None:
                collect(pending)
            pending = cur
            marks.append(time.perf_counter())
            c1 = counts()
            misses.append((c1[0] - c0[0], c1[1] - c0[1], round((tb - ta) * 1e3, 2), (c1[2] - c0[2]) >> 20,
                           (c1[3] - c0[3]) >> 20))
        collect(pending)

    # a few more untimed steps than the kernel leg: the first pipelined steps
    # still fill the device's cache of upload buffers (one 1 GiB and one
    # 256 MiB allocation show up as multi-millisecond host stalls).  The
    # timed region holds --e2e-steps (20) steps: the pipeline's fill (the
    # first upload) and drain (the last read-back), ~11 ms together, are
    # spread over them.
    run(max(1, args.warmup) + 3)
    gpu.wait()
    if dist is not None:
        dist.barrier()
    # Eight timed repetitions, the best reported (as for the CPU baseline):
    # on some machines a step's results arrive late every ~0.51 s of wall
    # time (from +3 ms to +125 ms over two or three iterations, no allocation,
    # pool growth, pinned-pool miss or garbage collection in them; the
    # device-timed leg never shows it), so a repetition of ~0.3 s can fall
    # between two of them where one of 30 steps (~0.5 s) could not.
    reps = []
    e2e_clocks = ClockSampler(os.environ.get("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", "0")).split(",")[0])
    e2e_clocks.start()
    for _ in range(8):
        t0 = time.perf_counter()
        marks.clear()
        misses.clear()
        gcs.clear()
        gc.callbacks.append(on_gc)
        run(args.e2e_steps)
        gc.callbacks.remove(on_gc)
        gpu.wait()
        dt_rep = (time.perf_counter() - t0) / args.e2e_steps
        # host time of each iteration (issue step i+1, read step i), for spotting stalls
        reps.append((dt_rep, [round((b - a) * 1e3, 2) for a, b in zip([t0] + marks[:-1], marks)], list(misses),
                     [g for g in gcs if g[2] >= 1.0]))
    e2e_clk = e2e_clocks.stop()
    dt_best, step_ms, step_misses, step_gcs = min(reps, key=lambda r: r[0])
    dt = max_over_ranks(dt_best, dist)
    return {"value": round(world * nbytes / dt / 1e9, 1), "unit": "GB/s", "ms_per_step": round(dt * 1e3, 3),
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps,
            "iteration_ms": step_ms, "repetitions_ms": [round(r[0] * 1e3, 3) for r in reps],
            "iteration_pinned_device_allocations_issue_ms_pool_growth_mib": step_misses,
            "gc_over_1ms": step_gcs, "clocks": e2e_clk,
            "api": "vulkpy_gb300 public API (Array(data=pinned), ops, Array.prefetch, np.asarray); "
                   "step i+1 issued before step i's results are read; best of 8 timed repetitions"}


# ---------------------------------------------------------------- matmul / MLP
def matmul_study(vk, gpu, timer, sizes=(1024, 4096, 8192), precisions=("fp32", "bf16", "bf16x3")):
    """C = A @ B, A, B ~ N(0,1) fp32 (seed 0), in fp32 SIMT, bf16 and split
    bf16x3 on tensor cores: TFLOP/s (2MNK / CUDA-event time) and relative
    Frobenius error of the whole product vs float64."""
    out = {}
    for n in sizes:
        rng = np.random.default_rng(0)
        A = rng.standard_normal((n, n), dtype=np.float32)
        B = rng.standard_normal((n, n), dtype=np.float32)
        ref = A.astype(np.float64) @ B.astype(np.float64)
        a, b = vk.Array(gpu, data=A), vk.Array(gpu, data=B)
        for prec in precisions:
            c = vk.vkarray.matmul(a, b, precision=prec)
            gpu.wait()
            reps = 3 if (prec == "fp32" and n >= 8192) else 10
            t0 = timer.mark()
            for _ in range(reps):
                c = vk.vkarray.matmul(a, b, precision=prec)
            t1 = timer.mark()
            gpu.wait()
            ms = timer.ms(t0, t1) / reps
            timer.free(t0, t1)
            err = float(np.linalg.norm(np.asarray(c) - ref) / np.linalg.norm(ref))
            out[f"{prec}_{n}"] = {"tflops": round(2 * n ** 3 / (ms * 1e-3) / 1e12, 1), "ms": round(ms, 3),
                                  "rel_err_fp64": float(f"{err:.3g}")}
        del a, b, c
    # 1-D @ 2-D: (8192,) @ (8192, 8192), an HBM-bound matrix-vector product
    # (fp32 GEMV for every precision); GB/s counts the matrix once
    n = sizes[-1]
    rng = np.random.default_rng(0)
    v = rng.standard_normal(n, dtype=np.float32)
    B = rng.standard_normal((n, n), dtype=np.float32)
    ref = v.astype(np.float64) @ B.astype(np.float64)
    a, b = vk.Array(gpu, data=v), vk.Array(gpu, data=B)
    c = a @ b
    gpu.wait()
    t0 = timer.mark()
    for _ in range(10):
        c = a @ b
    t1 = timer.mark()
    gpu.wait()
    ms = timer.ms(t0, t1) / 10
    timer.free(t0, t1)
    err = float(np.linalg.norm(np.asarray(c) - ref) / np.linalg.norm(ref))
    out[f"gemv_1d_{n}"] = {"gbs": round(4 * n * n / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 4),
                           "tflops": round(2 * n * n / (ms * 1e-3) / 1e12, 2), "rel_err_fp64": float(f"{err:.3g}")}
    del a, b, c
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak = json.load(open(peaks_path))["bf16_tflops"] if os.path.exists(peaks_path) else 1900.0
    best = out.get(f"bf16x3_{sizes[-1]}", {}).get("tflops")
    base = out.get(f"fp32_{sizes[-1]}", {}).get("tflops")
    return {"unit": "TFLOP/s (2MNK)", "results": out, "bf16_peak_tflops": peak,
            "bf16x3_vs_fp32_speedup": round(best / base, 2) if best and base else None,
            "note": "bf16x3 issues 3 tensor products per K step; TFLOP/s counts the algorithmic 2MNK"}


def mlp_study(vk, gpu, timer, steps=50, precisions=("fp32", "bf16x3")):
    """One Sequence.train step of Dense 784-1024, ReLU, Dense 1024-1024,
    Sigmoid, Dense 1024-10, softmax cross entropy, Adam(1e-3), batch 256,
    HeNormal(seed 1); steps/s for fp32 SIMT vs split-bf16x3 matmuls."""
    nn = vk.nn
    rng = np.random.default_rng(1)
    X = rng.standard_normal((256, 784)).astype(np.float32)
    Y = np.eye(10, dtype=np.float32)[rng.integers(0, 10, 256)]
    res = {}
    for prec in precisions:
        gpu.matmul_precision = prec
        opt = nn.Adam(gpu, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8)
        net = nn.Sequence([
            nn.Dense(gpu, 784, 1024, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 784, seed=1)),
            nn.ReLU(),
            nn.Dense(gpu, 1024, 1024, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 1024, seed=1)),
            nn.Sigmoid(),
            nn.Dense(gpu, 1024, 10, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 1024, seed=1)),
        ], nn.SoftmaxCrossEntropyLoss())
        x, y = vk.Array(gpu, data=X), vk.Array(gpu, data=Y)
        for _ in range(5):
            net.train(x, y)
        gpu.wait()
        t0 = timer.mark()
        for _ in range(steps):
            _, loss = net.train(x, y)
        t1 = timer.mark()
        gpu.wait()
        ms = timer.ms(t0, t1) / steps
        timer.free(t0, t1)
        res[prec] = {"steps_per_s": round(1000.0 / ms, 1), "ms_per_step": round(ms, 4),
                     "loss_after": float(np.asarray(loss))}
        # the same step captured once as a CUDA graph and replayed
        step = net.compile(x, y)
        for _ in range(3):
            step()
        gpu.wait()
        t0 = timer.mark()
        for _ in range(steps * 4):
            _, loss = step()
        t1 = timer.mark()
        gpu.wait()
        ms = timer.ms(t0, t1) / (steps * 4)
        timer.free(t0, t1)
        res[prec + "_graph"] = {"steps_per_s": round(1000.0 / ms, 1), "ms_per_step": round(ms, 4),
                                "loss_after": float(np.asarray(loss))}
        del step, net, opt
    gpu.matmul_precision = "fp32"
    flop = 3 * 2 * 256 * (784 * 1024 + 1024 * 1024 + 1024 * 10)
    res["flop_per_step"] = flop
    for k in list(res):
        if isinstance(res[k], dict):
            res[k]["tflops"] = round(flop * res[k]["steps_per_s"] / 1e12, 2)
    # roofline of the fastest mode: algorithmic FLOP against the bf16 peak and
    # the Adam update's 28 B/parameter against the copy peak (latency-bound:
    # ~25 launches per step, each far below either roof)
    best = max((v for v in res.values() if isinstance(v, dict)), key=lambda v: v["steps_per_s"])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    pk = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {"bf16_tflops": 1900.0, "hbm_gbs": 6800.0}
    params = 784 * 1024 + 1024 + 1024 * 1024 + 1024 + 1024 * 10 + 10
    res["roofline"] = {"bound": "latency", "steps_per_s": best["steps_per_s"],
                       "flop_frac": round(best["tflops"] / pk["bf16_tflops"], 4),
                       "adam_bytes_per_step": 28 * params,
                       "byte_frac": round(28 * params * best["steps_per_s"] / 1e9 / pk["hbm_gbs"], 4)}
    if "fp32" in res and "bf16x3" in res:
        res["speedup_bf16x3_graph_vs_fp32_eager"] = round(res["bf16x3_graph"]["steps_per_s"] /
                                                          res["fp32"]["steps_per_s"], 2)
        res["speedup_bf16x3_graph_vs_fp32_graph"] = round(res["bf16x3_graph"]["steps_per_s"] /
                                                          res["fp32_graph"]["steps_per_s"], 2)
    return res


def batched_study(vk, gpu, timer, n_models=64, steps=10, precisions=("fp32", "bf16x3")):
    """64 independent 2-layer MLPs of uneven sizes (seed 2: input width in
    [17,1021], hidden in [32,2048], output in [2,64], batch in [1,512]),
    Dense-ReLU-Dense, MSE loss, SGD(1e-2).  One step trains all 64 models.
    Compared: the per-op eager path (fp32, one stream), the whole step
    captured in one CUDA graph with one parallel branch per model, and the
    grouped step (nn.GroupedSequence: one persistent grouped GEMM per layer
    and direction for all 64 models, grouped loss / bias-gradient / SGD
    kernels), eager and captured; fp32 SIMT and split-bf16x3 tensor cores."""
    nn = vk.nn
    rng = np.random.default_rng(2)
    dims = []
    for _ in range(n_models):
        i_ = int(rng.integers(17, 1022)); h_ = int(rng.integers(32, 2049))
        o_ = int(rng.integers(2, 65)); b_ = int(rng.integers(1, 513))
        dims.append((i_, h_, o_, b_))
    data = [(rng.standard_normal((b, i)).astype(np.float32), rng.standard_normal((b, o)).astype(np.float32))
            for i, h, o, b in dims]
    flop = sum(6 * b * (i * h + h * o) for i, h, o, b in dims)

    def build(seed0):
        nets = []
        for k, (i, h, o, b) in enumerate(dims):
            opt = nn.SGD(lr=1e-2)
            nets.append(nn.Sequence([
                nn.Dense(gpu, i, h, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, i, seed=seed0 + k)),
                nn.ReLU(),
                nn.Dense(gpu, h, o, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, h, seed=seed0 + 1000 + k)),
            ], nn.MSELoss()))
        return nets

    arrays = [(vk.Array(gpu, data=x), vk.Array(gpu, data=y)) for x, y in data]
    res = {"models": n_models, "flop_per_step": flop}

    def timed(fn, reps):
        gpu.wait()
        t0 = timer.mark()
        for _ in range(reps):
            fn()
        t1 = timer.mark()
        gpu.wait()
        ms = timer.ms(t0, t1) / reps
        timer.free(t0, t1)
        return {"steps_per_s": round(1000.0 / ms, 1), "ms_per_step": round(ms, 3),
                "tflops": round(flop / (ms * 1e-3) / 1e12, 2)}

    for prec in precisions:
        gpu.matmul_precision = prec
        nets = build(7)
        def eager():
            for net, (x, y) in zip(nets, arrays):
                net.train(x, y)
        eager()
        if prec == "fp32":
            res["eager_fp32"] = timed(eager, steps)
        g = vk.graph.Graph(gpu)
        with g:
            for net, (x, y) in zip(nets, arrays):
                with gpu.branch():
                    net.train(x, y)
        g.launch()
        res[f"graph_{prec}"] = timed(g.launch, steps * 5)
        del g, nets
        # grouped: one launch per layer and direction for all 64 models
        nets = build(7)
        grp = nn.GroupedSequence(nets)
        xs = [x for x, _ in arrays]
        ys = [y for _, y in arrays]
        grp.train(xs, ys)
        res[f"grouped_eager_{prec}"] = timed(lambda: grp.train(xs, ys), steps)
        g = vk.graph.Graph(gpu)
        with g:
            grp.train(xs, ys)
        g.launch()
        res[f"grouped_graph_{prec}"] = timed(g.launch, steps * 5)
        del g, grp, nets
    gpu.matmul_precision = "fp32"
    if "eager_fp32" in res and "graph_bf16x3" in res:
        res["speedup_graph_bf16x3_vs_eager_fp32"] = round(res["graph_bf16x3"]["steps_per_s"] /
                                                          res["eager_fp32"]["steps_per_s"], 2)
        res["speedup_grouped_graph_bf16x3_vs_eager_fp32"] = round(res["grouped_graph_bf16x3"]["steps_per_s"] /
                                                                  res["eager_fp32"]["steps_per_s"], 2)
    return res


def reduction_precision_study(vk, gpu, timer, n=1 << 28):
    """sum of 2^28 float32 values 1e6*N(0,1) + U[0,1) (generated on the GPU
    by Xoshiro128pp seed 0), in the three summation modes, against a float64
    sum of the same float32 values; plus the time of each mode."""
    from vulkpy_gb300 import _lib
    import ctypes
    r = vk.random.Xoshiro128pp(gpu, size=1 << 20, seed=0)
    z = r.normal(shape=(n,), mean=0.0, stddev=1e6)
    u = r.random(shape=(n,))
    x = z + u
    del z, u
    host = np.asarray(x)
    truth = float(np.sum(host, dtype=np.float64))
    scale = float(np.sum(np.abs(host), dtype=np.float64))
    out = vk.Array(gpu, shape=(1,))
    res = {"n": n, "truth_fp64": truth, "sum_abs": scale}
    for name, mode in (("plain", _lib.RED_PLAIN), ("pairwise", _lib.RED_PAIRWISE),
                       ("compensated", _lib.RED_COMPENSATED)):
        def run():
            check = _lib.check
            check(_lib.lib.vkc_reduce_all(gpu.handle, _lib.SUM, mode, x._dptr(), n, out._buf.ptr, ctypes.c_float(1.0)))
        run()
        gpu.wait()
        t0 = timer.mark()
        for _ in range(5):
            run()
        t1 = timer.mark()
        gpu.wait()
        ms = timer.ms(t0, t1) / 5
        timer.free(t0, t1)
        out._written()
        v = float(np.asarray(out)[0])
        res[name] = {"value": v, "abs_err": abs(v - truth), "err_rel_sum_abs": abs(v - truth) / scale,
                     "gbs": round(4 * n / (ms * 1e-3) / 1e9, 1)}
    return res


def chain32(x, y):
    """A fixed 32-op elementwise chain over two same-shape arrays."""
    t = x * 1.0001 + y
    t = t.tanh()
    t = t * y - 0.5
    t = t.exp()
    t = t.max(0.25).min(4.0)
    t = t.log() * 0.5
    t = t + x * 0.125
    t = t.sin() * t.cos()
    t = t / (y.abs() + 1.0)
    t = t.clamp(-2.0, 2.0)
    t = t ** 2.0 + 1.0
    t = t.sqrt() - x
    t = t.atan() * 2.0
    t = (t - y) * (t + y)
    t = t.tanh() + t.sign()
    return t * 0.5


def small_suite_study(vk, gpu, timer, reps=100):
    """The plain-fp32 small op suite (numpy seed 0, in this order): A (512,1024)
    and B (1,1024) uniform[-1,1); M1, M2 (256,256) N(0,1); 4096 indices in
    [0, 524288); Xoshiro128pp(size 64, seed 0) with 65536 uniforms and 65536
    normals.  Latency-bound, so per op:
      api_us     host wall time per call through the public API (calls back
                 to back, one wait at the end: launch cost included);
      device_us  device time per call, the calls captured in a CUDA graph and
                 replayed (CUDA events), i.e. without host launch cost;
      oracle_us  the oracle's C restatement of the shader on all host
                 threads (the reference's own CPU path is unavailable);
      numpy_us   numpy, where numpy has the op."""
    import time as _time
    from oracle import ops as O  # CPU baseline column only
    L = O.lib()
    rng = np.random.default_rng(0)
    A_ = rng.uniform(-1, 1, size=(512, 1024)).astype(np.float32)
    B_ = rng.uniform(-1, 1, size=(1, 1024)).astype(np.float32)
    M1 = rng.standard_normal((256, 256)).astype(np.float32)
    M2 = rng.standard_normal((256, 256)).astype(np.float32)
    idx = rng.integers(0, 524288, 4096).astype(np.uint32)
    a, b = vk.Array(gpu, data=A_), vk.Array(gpu, data=B_)
    m1, m2 = vk.Array(gpu, data=M1), vk.Array(gpu, data=M2)
    ix = vk.U32Array(gpu, data=idx)
    r = vk.random.Xoshiro128pp(gpu, size=64, seed=0)
    ops = {
        "A+B": lambda: a + b, "A*B": lambda: a * b, "A/(|B|+1)": lambda: a / (b.abs() + 1.0),
        "A**2": lambda: a ** 2.0, "exp(A)": lambda: a.exp(), "tanh(A)": lambda: a.tanh(),
        "clamp(A,-.5,.5)": lambda: a.clamp(-0.5, 0.5),
        "sum0": lambda: a.sum(axis=0), "sum1": lambda: a.sum(axis=1), "sum": lambda: a.sum(),
        "mean0": lambda: a.mean(axis=0), "mean1": lambda: a.mean(axis=1), "mean": lambda: a.mean(),
        "max0": lambda: a.maximum(axis=0), "max1": lambda: a.maximum(axis=1), "max": lambda: a.maximum(),
        "M1@M2": lambda: m1 @ m2, "gather4096": lambda: a.gather(ix),
        "random65536": lambda: r.random(shape=(65536,)), "normal65536": lambda: r.normal(shape=(65536,)),
    }
    p = lambda x: x.ctypes.data
    sa, sb = np.array([512, 1024], np.int64), np.array([1, 1024], np.int64)
    out = np.empty_like(A_)
    r0, r1 = np.empty(1024, np.float32), np.empty(512, np.float32)
    st = O.Xoshiro128pp(0, 64)
    u = np.empty(65536, np.float32)
    oracle = {
        "A+B": lambda: L.bcast_binary(0, p(A_), p(sa), p(B_), p(sb), p(out), p(sa), 2),
        "A*B": lambda: L.bcast_binary(2, p(A_), p(sa), p(B_), p(sb), p(out), p(sa), 2),
        "exp(A)": lambda: L.ew_unary(14, p(A_), p(out), A_.size),
        "tanh(A)": lambda: L.ew_unary(10, p(A_), p(out), A_.size),
        "A**2": lambda: L.ew_scalar(4, p(A_), np.float32(2.0), p(out), A_.size),
        "sum0": lambda: L.reduce_axis(0, p(A_), 1, 512, 1024, p(r0)),
        "sum1": lambda: L.reduce_axis(0, p(A_), 512, 1024, 1, p(r1)),
        "sum": lambda: L.reduce_all(0, p(A_), A_.size),
        "max0": lambda: L.reduce_axis(2, p(A_), 1, 512, 1024, p(r0)),
        "max1": lambda: L.reduce_axis(2, p(A_), 512, 1024, 1, p(r1)),
        "M1@M2": lambda: O.matmul(M1, M2),
        "gather4096": lambda: O.gather(A_.reshape(-1), idx),
        "random65536": lambda: L.xo_generate(p(st.state), 64, p(u), 65536, 1),
        "normal65536": lambda: st.normal(65536),
    }
    npy = {
        "A+B": lambda: A_ + B_, "A*B": lambda: A_ * B_, "A/(|B|+1)": lambda: A_ / (np.abs(B_) + np.float32(1)),
        "A**2": lambda: A_ * A_, "exp(A)": lambda: np.exp(A_), "tanh(A)": lambda: np.tanh(A_),
        "clamp(A,-.5,.5)": lambda: np.clip(A_, -0.5, 0.5), "sum0": lambda: A_.sum(axis=0),
        "sum1": lambda: A_.sum(axis=1), "sum": lambda: A_.sum(), "max0": lambda: A_.max(axis=0),
        "max1": lambda: A_.max(axis=1), "max": lambda: A_.max(), "M1@M2": lambda: M1 @ M2,
        "gather4096": lambda: A_.reshape(-1)[idx],
    }

    def host_us(fn, n):
        fn()
        t0 = _time.perf_counter()
        for _ in range(n):
            fn()
        return (_time.perf_counter() - t0) / n * 1e6

    res = {}
    for name, fn in ops.items():
        for _ in range(3):
            fn()
        gpu.wait()
        t0 = _time.perf_counter()
        keep = [fn() for _ in range(reps)]
        gpu.wait()
        api = (_time.perf_counter() - t0) / reps * 1e6
        del keep
        g = vk.graph.Graph(gpu)
        with g:
            keep = [fn() for _ in range(reps)]
        g.launch()
        gpu.wait()
        t0 = timer.mark()
        g.launch()
        t1 = timer.mark()
        gpu.wait()
        dev = timer.ms(t0, t1) / reps * 1e3
        timer.free(t0, t1)
        del g, keep
        row = {"api_us": round(api, 2), "device_us": round(dev, 2)}
        if name in oracle:
            row["oracle_us"] = round(host_us(oracle[name], 20), 1)
        if name in npy:
            row["numpy_us"] = round(host_us(npy[name], 20), 1)
        res[name] = row
    return {"ops": res, "reps": reps, "oracle_threads": int(L.oracle_threads()),
            "note": "latency suite: parity with the reference is checked by tests/test_gpu_golden.py (small_suite_*)"}


def train_loop_study(vk, gpu, epochs=100, batch=32):
    """The classification example's loop (4-128-128-3, ReLU, Softmax,
    CrossEntropyLoss(sum), Adam lr 1e-4, batch 32, 100 epochs, 120/30 split)
    on a synthetic Iris-shaped set (3 Gaussian classes of 50 rows in 4-D,
    numpy seed 0).  Each epoch reads back the train loss and the test-set
    class predictions, as the example prints them.  Three loops:
      host:   numpy shuffle, one upload per batch, numpy argmax (the
              example's own structure);
      device: data resident, device permutation + row gathers, device argmax;
      graph:  the device epoch captured once and replayed."""
    import time as _time
    nn = vk.nn
    rng = np.random.default_rng(0)
    means = rng.uniform(1.0, 7.0, size=(3, 4))
    x = np.concatenate([rng.normal(means[c], 0.45, size=(50, 4)) for c in range(3)]).astype(np.float32)
    lab = np.repeat(np.arange(3), 50)
    order = rng.permutation(150)
    x, lab = x[order], lab[order]
    y = np.identity(3, dtype=np.float32)[lab]
    tx, ty, vx, vlab = x[:120], y[:120], x[120:], lab[120:]

    def make():
        opt = nn.Adam(gpu, lr=1e-4)
        return nn.Sequence([
            nn.Dense(gpu, 4, 128, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 4, seed=1)), nn.ReLU(),
            nn.Dense(gpu, 128, 128, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 128, seed=2)), nn.ReLU(),
            nn.Dense(gpu, 128, 3, w_opt=opt, b_opt=opt, w_init=nn.HeNormal(gpu, 128, seed=3)), nn.Softmax(),
        ], nn.CrossEntropyLoss(reduce="sum"))

    res = {"epochs": epochs, "batch": batch, "rows": 120, "data": "synthetic Iris-shaped (numpy seed 0)"}
    VX = vk.Array(gpu, data=vx)

    # host loop
    net = make()
    hrng = np.random.default_rng(1)
    idx = np.arange(120)
    gpu.wait()
    t0 = _time.perf_counter()
    for _ in range(epochs):
        hrng.shuffle(idx)
        total = vk.Array(gpu, shape=(1,))
        total[:] = 0
        for s in range(0, 120, batch):
            b = idx[s:s + batch]
            _, loss = net.train(vk.Array(gpu, data=tx[b]), vk.Array(gpu, data=ty[b]))
            total += loss
        pred = np.argmax(np.asarray(net.predict(VX)), axis=1)
        float(np.asarray(total)[0])
    dt = _time.perf_counter() - t0
    res["host"] = {"epochs_per_s": round(epochs / dt, 1), "accuracy": float(np.mean(pred == vlab))}

    X, Y = vk.Array(gpu, data=tx), vk.Array(gpu, data=ty)

    def epoch(net, r):
        total = vk.zeros(gpu, shape=(1,))
        for xb, yb in nn.minibatches(X, Y, batch, rng=r):
            _, loss = net.train(xb, yb)
            total += loss
        return total, net.predict(VX).argmax(axis=1)

    net, r = make(), vk.random.Xoshiro128pp(gpu, seed=1)
    epoch(net, r)   # builds the row-range tables
    gpu.wait()
    t0 = _time.perf_counter()
    for _ in range(epochs):
        total, cls = epoch(net, r)
        float(np.asarray(total)[0])
        pred = np.asarray(cls)
    dt = _time.perf_counter() - t0
    res["device"] = {"epochs_per_s": round(epochs / dt, 1), "accuracy": float(np.mean(pred == vlab))}

    net, r = make(), vk.random.Xoshiro128pp(gpu, seed=1)
    epoch(net, r)
    g = vk.graph.Graph(gpu)
    with g:
        total, cls = epoch(net, r)
    g.launch()
    gpu.wait()
    t0 = _time.perf_counter()
    for _ in range(epochs):
        g.launch()
        float(np.asarray(total)[0])
        pred = np.asarray(cls)
    dt = _time.perf_counter() - t0
    res["graph"] = {"epochs_per_s": round(epochs / dt, 1), "accuracy": float(np.mean(pred == vlab))}
    res["speedup_graph_vs_host"] = round(res["graph"]["epochs_per_s"] / res["host"]["epochs_per_s"], 2)
    del g
    return res


def chain_study(vk, gpu, timer, n=4096, reps=20):
    """The 32-op chain on (4096, 4096) fp32: op by op (32 launches, every
    intermediate written and re-read) vs one fused kernel (reads x, y once,
    writes the result once); results must be bit-identical."""
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, n), dtype=np.float32)
    Y = rng.uniform(0.5, 2.0, (n, n)).astype(np.float32)
    x, y = vk.Array(gpu, data=X), vk.Array(gpu, data=Y)
    fused = vk.fusion.fuse(chain32)
    a = chain32(x, y)
    b = fused(x, y)
    same = bool(np.array_equal(np.asarray(a), np.asarray(b)))
    ops = fused.source(x, y).count("const float t")
    out = {"shape": [n, n], "ops": ops, "bit_identical": same}
    for label, fn in (("per_op", lambda: chain32(x, y)), ("fused", lambda: fused(x, y))):
        fn()
        gpu.wait()
        t0 = timer.mark()
        for _ in range(reps):
            r = fn()
        t1 = timer.mark()
        gpu.wait()
        ms = timer.ms(t0, t1) / reps
        timer.free(t0, t1)
        out[label] = {"ms": round(ms, 4), "io_gbs": round(12 * n * n / (ms * 1e-3) / 1e9, 1)}
    out["speedup"] = round(out["per_op"]["ms"] / out["fused"]["ms"], 2)
    out["note"] = "io_gbs counts the fused kernel's 12 B/element (x, y in, result out) for both"
    return out


# ---------------------------------------------------------------- CPU oracle
def cpu_suite_pass(O, X, row, col, idx, st, sizes):
    """The same step on the CPU restatement (oracle/vkoracle.c), OpenMP."""
    L = O.lib()
    p = lambda a: a.ctypes.data
    rows, cols = X.shape
    n = X.size
    out = np.empty_like(X)
    sa = np.array([rows, cols], np.int64)
    for other in (row, col):
        so = np.array(other.shape, np.int64)
        for op in range(7):
            L.bcast_binary(op, p(X), p(sa), p(other), p(so), p(out), p(sa), 2)
    Z = np.empty_like(X)
    L.ew_unary(0, p(X), p(Z), n)
    L.ew_scalar(0, p(Z), np.float32(1e-3), p(Z), n)
    for op in (18, 19, 15):
        L.ew_unary(op, p(Z), p(out), n)
    L.ew_unary(18, p(Z), p(Z), n)
    E = np.empty_like(X)
    L.ew_scalar(2, p(X), np.float32(1e-4), p(E), n)
    L.ew_unary(14, p(E), p(E), n)
    r0 = np.empty(cols, np.float32)
    r1 = np.empty(rows, np.float32)
    for src, ops in ((X, (0, 2, 3, 0)), (E, (1,))):
        for op in ops:
            L.reduce_axis(op, p(src), 1, rows, cols, p(r0))
            L.reduce_axis(op, p(src), rows, cols, 1, p(r1))
            L.reduce_all(op, p(src), n)
    g = np.empty(idx.size, np.float32)
    L.gather(p(X), n, p(idx), idx.size, p(g))
    states, m = sizes
    L.xo_generate(p(st), states, p(out), n, 1)
    L.xo_generate(p(st), states, p(out), n, 1)
    L.box_muller(p(out), p(out), n, np.float32(0), np.float32(1))
    L.xo_generate(p(st), states, p(out), n, 0)
    for other in (row, col):
        so = np.array(other.shape, np.int64)
        for op in range(4):
            L.bcast_binary(op, p(X), p(sa), p(other), p(so), p(X), p(sa), 2)


def cpu_sample(args):
    """A bounded sample of the workload: the first `rows` rows, indices and
    PRNG states scaled by the same factor."""
    rows = args.cpu_rows
    frac = rows / args.rows
    X, row, col, idx = make_inputs(args.rows, args.cols, args.n_idx)
    Xs = np.ascontiguousarray(X[:rows])
    cols_ = np.ascontiguousarray(col[:rows])
    n_idx = int(args.n_idx * frac)
    idxs = np.ascontiguousarray(idx[:n_idx] % np.uint32(Xs.size))
    states = max(1, int(args.states * frac))
    del X
    return Xs, row, cols_, idxs, states, n_idx


_CPU_CACHE = {}


def _cpu_data(args):
    from oracle import ops as O  # checker / CPU baseline only
    if "data" not in _CPU_CACHE:
        Xs, row, col, idx, states, n_idx = cpu_sample(args)
        _CPU_CACHE["data"] = (Xs, row, col, idx, O.Xoshiro128pp(0, states).state, states, n_idx)
    return _CPU_CACHE["data"]


def cpu_measure_once(args) -> float:
    from oracle import ops as O
    Xs, row, col, idx, st, states, n_idx = _cpu_data(args)
    t0 = time.perf_counter()
    cpu_suite_pass(O, Xs, row, col, idx, st, (states, 0))
    return time.perf_counter() - t0


def cpu_info(args):
    import oracle
    Xs, row, col, idx, st, states, n_idx = _cpu_data(args)
    return step_bytes(Xs.shape[0], Xs.shape[1], n_idx, states), oracle.lib().oracle_threads(), Xs.shape


def cpu_baseline(args):
    nbytes, threads, shape = cpu_info(args)
    cpu_measure_once(args)  # warm-up
    times = [cpu_measure_once(args) for _ in range(args.cpu_passes)]
    best = min(times)
    return {"value": round(nbytes / best / 1e9, 2), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{shape[0]} of {args.rows} rows ({shape[0] * shape[1] * 4 / 2**20:.0f} MiB), indices and "
                      f"PRNG states scaled alike; best of {len(times)} passes of the step on the CPU restatement "
                      f"of the reference's shaders (oracle/vkoracle.c, OpenMP)"}


def reference_arm(args, rank, world):
    if rank != 0:
        return None
    nbytes, threads, shape = cpu_info(args)
    for _ in range(args.warmup):
        cpu_measure_once(args)
    times = [cpu_measure_once(args) for _ in range(args.steps)]
    dt = float(np.mean(times))
    value = nbytes / dt / 1e9
    sample = (f"{shape[0]} of {args.rows} rows per step, indices and PRNG states scaled alike; "
              f"CPU restatement of the reference's shaders (oracle/vkoracle.c), OpenMP over all host threads")
    return {"metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (numpy default_rng seed 0)",
            "impl": "reference",
            "config": {"workload": f"bandwidth suite, bounded sample on host cores ({shape[0]}x{shape[1]})",
                       "bytes_per_step": nbytes},
            "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_study(args):
    import vulkpy_gb300 as vk
    gpu = vk.GPU(0)
    timer = Timer(vk, gpu)
    if args.study == "matmul":
        return matmul_study(vk, gpu, timer, sizes=tuple(int(x) for x in args.mm_sizes.split(",")),
                            precisions=tuple(args.mm_precisions.split(",")))
    if args.study == "mlp":
        return mlp_study(vk, gpu, timer, precisions=tuple(args.mm_precisions.split(",")))
    if args.study == "batched":
        return batched_study(vk, gpu, timer, precisions=tuple(args.mm_precisions.split(",")))
    fn = {"batched": batched_study, "chain": chain_study,
          "reduction_precision": reduction_precision_study, "small_suite": small_suite_study}.get(args.study)
    if fn is None:
        return train_loop_study(vk, gpu)
    return fn(vk, gpu, timer)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rows", type=int, default=ROWS)
    ap.add_argument("--cols", type=int, default=COLS)
    ap.add_argument("--n-idx", type=int, default=N_IDX)
    ap.add_argument("--states", type=int, default=PRNG_STATES)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-rows", type=int, default=2048)
    ap.add_argument("--cpu-passes", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the matmul and MLP studies")
    ap.add_argument("--study", default=None,
                    choices=["matmul", "mlp", "batched", "chain", "reduction_precision", "train_loop", "small_suite"],
                    help="run only this study (a small case for profiling) and print its JSON")
    ap.add_argument("--mm-sizes", default="1024,4096,8192", help="matmul study sizes, comma separated")
    ap.add_argument("--mm-precisions", default="fp32,bf16,bf16x3", help="matmul study precisions")
    args = ap.parse_args()
    if args.study is not None:
        print(json.dumps(run_study(args)), flush=True)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        tdist.init_process_group("gloo")
        dist = tdist

    if args.impl == "reference":
        res = reference_arm(args, rank, world)
        if res is not None:
            print(json.dumps(res), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    res = gpu_arm(args, rank, world, dist)
    if rank == 0:
        if not args.no_cpu:
            res["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(res), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
