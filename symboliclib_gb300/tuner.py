"""Schedule autotuner and learned schedule proposer.

The schedule of a unit (executor, launch structure, fusion depth, block size,
work items per thread, tile size) changes only speed, never values.
`exhaustive` times every schedule in `SPACE` on the GPU and returns the
fastest; a compiled-executor schedule is compiled (NVRTC) the first time it
is timed, and that compile time counts as tuning time.  `CostModel` is an MLP
(the engine's FP32 kernels, native.MLP) that predicts the log run time of a
unit under a schedule from plan features; `tune_with_model` times the
default schedule and the model's k - 1 best-ranked others, so tuning costs k
timings (and at most k compiles) instead of len(SPACE).  The training data
are timings the tuner itself collected."""
from __future__ import annotations

import ctypes as C
import itertools
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import native

KINDS = {"plain": (native.SCHEDULE_PLAIN, 0), "levels": (native.SCHEDULE_LEVELS, 0),
         "fused2": (native.SCHEDULE_LEVELS, 2), "persistent": (native.SCHEDULE_PERSISTENT, 0)}


EXECUTORS = {"compiled": native.EXEC_COMPILED, "interpreter": native.EXEC_INTERPRETER}


@dataclass(frozen=True)
class Sched:
    kind: str
    items: int
    tpb: int
    tile: int  # interpreter: a tile is (tpb / lanes) * items * tile work items
    lanes: int = 1  # interpreter only
    executor: str = "interpreter"

    def apply(self, unit: native.Unit, math_mode: int = native.MATH_FAST, graph: int = 1) -> None:
        k, depth = KINDS[self.kind]
        unit.set_schedule(kind=k, math=math_mode, threads_per_block=self.tpb,
                          items_per_tile=self.tpb // self.lanes * self.items * self.tile, items_per_thread=self.items,
                          use_graph=graph, fusion_depth=depth, lanes_per_item=self.lanes,
                          executor=EXECUTORS[self.executor])


# (items per thread, lanes per item): several items per thread for small
# register files, several lanes per item for large ones
SHAPES = ((1, 1), (2, 1), (4, 1), (1, 2), (1, 4))
INTERPRETER_SPACE = [Sched(k, i, t, f, l) for k, (i, l), t, f in
                     itertools.product(KINDS, SHAPES, (64, 128, 256), (1, 4))]
# The compiled executor has no tiles, lanes or fusion depth: kind x items x tpb.
COMPILED_SPACE = [Sched(k, i, t, 1, 1, "compiled") for k, i, t in
                  itertools.product(("plain", "levels", "persistent"), (1, 2, 4), (64, 128, 256))]
SPACE = COMPILED_SPACE + INTERPRETER_SPACE
DEFAULT = Sched("levels", 1, 128, 1, 1, "compiled")


def time_schedule(unit: native.Unit, sched: Sched, stream, flush=None, runs: int = 5, warmup: int = 2) -> float:
    """Median microseconds of one run under `sched` (CUDA events on the unit's stream)."""
    import torch
    sched.apply(unit)
    lib = native.symgb()
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            native.check(lib.symgb_run_async(unit.handle))
        ts = []
        for _ in range(runs):
            if flush is not None:
                flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            native.check(lib.symgb_run_async(unit.handle))
            b.record(stream)
            ts.append((a, b))
        torch.cuda.synchronize()
    native.check(lib.symgb_synchronize(unit.handle))
    return float(np.median([a.elapsed_time(b) for a, b in ts]) * 1e3)


def bind_stream(unit: native.Unit):
    import torch
    stream = torch.cuda.Stream()
    native.check(native.symgb().symgb_set_stream(unit.handle, C.c_void_p(stream.cuda_stream)))
    return stream


@dataclass
class TuneResult:
    best: Sched
    best_us: float
    timings: dict = field(default_factory=dict)
    seconds: float = 0.0
    timed: int = 0


def exhaustive(unit: native.Unit, stream, flush=None, space=SPACE, runs: int = 5) -> TuneResult:
    t0 = time.perf_counter()
    timings = {}
    for s in space:
        try:
            timings[s] = time_schedule(unit, s, stream, flush, runs)
        except RuntimeError:
            continue  # schedule does not fit (e.g. register file too large)
    best = min(timings, key=timings.get)
    return TuneResult(best, timings[best], timings, time.perf_counter() - t0, len(timings))


# ------------------------------------------------------------------ features

def plan_features(stats: native.Stats, num_sets: int) -> np.ndarray:
    """Size and operation-mix features of a unit (log-scaled counts)."""
    lg = lambda v: math.log1p(float(v))
    S = max(1, num_sets)
    return np.array([
        lg(stats.num_outputs * S), lg(stats.num_intermediates * S), lg(stats.num_inputs * S),
        lg(stats.flops * S), lg((stats.divs + stats.sqrts) * S), lg(stats.gathers * S),
        lg(stats.index_entries), lg(stats.constant_entries), float(stats.num_kernels), float(stats.num_levels),
        float(stats.max_registers), lg(stats.program_words), lg(S),
        lg(stats.bundles * S), float(stats.bundle_entries) / max(1.0, float(stats.bundles)),
    ], np.float32)


def schedule_features(s: Sched) -> np.ndarray:
    onehot = [1.0 if s.kind == k else 0.0 for k in KINDS] + [1.0 if s.executor == "compiled" else 0.0]
    return np.array(onehot + [math.log2(s.lanes), math.log2(s.items), math.log2(s.tpb), math.log2(s.tile)], np.float32)


def features(stats: native.Stats, num_sets: int, s: Sched) -> np.ndarray:
    p = plan_features(stats, num_sets)
    q = schedule_features(s)
    # interactions: work per launch under this schedule
    # register file bytes per thread under this shape (occupancy)
    regfile = np.array([math.log2(1.0 + float(stats.max_registers) * s.items / s.lanes)], np.float32)
    compiled = 1.0 if s.executor == "compiled" else 0.0
    return np.concatenate([p, q, p[:6] * q[-3] / 8.0, p[:6] * q[-2] / 8.0, p[:6] * q[-4] / 8.0, regfile,
                           p[:6] * compiled, regfile * (1.0 - compiled)])


class CostModel:
    """MLP regression of log(run time in us) on `features`."""

    def __init__(self, hidden: int = 64, seed: int = 0):
        self.hidden, self.seed = hidden, seed
        self.net = None
        self.mu = self.sd = None

    def fit(self, X: np.ndarray, y_us: np.ndarray, epochs: int = 3000, lr: float = 3e-3) -> float:
        X = np.asarray(X, np.float32)
        self.mu, self.sd = X.mean(0), X.std(0) + 1e-6
        self.net = native.MLP(X.shape[1], self.hidden, self.seed)
        return self.net.train((X - self.mu) / self.sd, np.log(np.asarray(y_us, np.float32)), epochs, lr)

    def predict_us(self, X: np.ndarray) -> np.ndarray:
        X = np.asarray(X, np.float32)
        return np.exp(self.net.predict((X - self.mu) / self.sd))


def propose(model: CostModel, stats: native.Stats, num_sets: int, k: int = 3, space=SPACE,
            keep=DEFAULT) -> list[Sched]:
    """k schedules to time: `keep` (the default schedule; None for none) and
    the model's best-ranked others."""
    X = np.stack([features(stats, num_sets, s) for s in space])
    order = np.argsort(model.predict_us(X))
    picks = [keep] if keep is not None else []
    for i in order:
        if len(picks) >= k:
            break
        if space[i] != keep:
            picks.append(space[i])
    return picks


def tune_with_model(unit: native.Unit, model: CostModel, stream, flush=None, k: int = 3, runs: int = 5) -> TuneResult:
    t0 = time.perf_counter()
    timings = {}
    for s in propose(model, unit.stats(), unit.num_sets, k):
        try:
            timings[s] = time_schedule(unit, s, stream, flush, runs)
        except RuntimeError:
            continue
    best = min(timings, key=timings.get)
    return TuneResult(best, timings[best], timings, time.perf_counter() - t0, len(timings))


# ------------------------------------------------------- per-kernel shapes

# Launch shapes a single kernel can take: (items per thread, lanes per item)
# x threads per block.
KERNEL_SHAPES = [(i, l, t) for (i, l) in SHAPES for t in (64, 128, 256)]
COMPILED_KERNEL_SHAPES = [(i, 1, t) for i in (1, 2, 4) for t in (64, 128, 256)]

_OPNAMES = {5: "add", 6: "sub", 7: "mul", 8: "div", 9: "neg", 10: "sqrt", 11: "rec", 12: "fma", 23: "fma", 24: "fma",
            25: "fma", 26: "div", 27: "sqrt", 28: "rec"}


def program_summary(unit: native.Unit, k: int, math_mode: int = native.MATH_FAST) -> dict:
    """Operation counts of kernel k's device program (decoded bundles)."""
    lib = native.symgb()
    r, nl = C.c_int(), C.c_int()
    n = lib.symgb_kernel_program(unit.handle, k, math_mode, None, 0, C.byref(r), C.byref(nl))
    buf = (C.c_uint64 * n)()
    lib.symgb_kernel_program(unit.handle, k, math_mode, buf, n, C.byref(r), C.byref(nl))
    words = list(buf)
    pc, bundles, entries = nl.value, 0, 0
    counts = {"add": 0, "sub": 0, "mul": 0, "div": 0, "neg": 0, "sqrt": 0, "rec": 0, "fma": 0, "st": 0, "other": 0}
    while words[pc] & 0xff:
        op, cnt = words[pc] & 0xff, (words[pc] >> 8) & 0xffff
        counts["st" if op == 4 else _OPNAMES.get(op, "other")] += cnt
        bundles += 1
        entries += cnt
        pc += 1 + (cnt + 1) // 2
    ldx = sum(1 for w in words[:nl.value] if w & 0xff == 1)  # x gathers (OP_LDX)
    ldc = sum(1 for w in words[:nl.value] if w & 0xff == 2)  # constant-table reads (OP_LDC)
    return {"registers": r.value, "loads": nl.value, "ldx": ldx, "ldc": ldc, "bundles": bundles, "entries": entries,
            **counts}


def kernel_features(unit: native.Unit, k: int, num_sets: int, shape, summary: dict) -> np.ndarray:
    """Tree features of one kernel (its template program) and a launch shape."""
    items, lanes, tpb = shape
    lg = lambda v: math.log1p(float(v))
    work = unit.kernel_instances[k] * max(1, num_sets)
    sm = summary
    flops = sm["add"] + sm["sub"] + sm["mul"] + sm["neg"] + 2 * sm["fma"]
    base = np.array([lg(work), lg(sm["entries"]), lg(sm["loads"]), float(sm["registers"]) / 64.0, lg(sm["bundles"]),
                     sm["entries"] / max(1, sm["bundles"]), lg(flops), lg(sm["div"] + sm["rec"]), lg(sm["sqrt"]),
                     lg(sm["st"]), float(unit.kernel_levels[k])], np.float32)
    shp = np.array([math.log2(items), math.log2(lanes), math.log2(tpb) - 6.0], np.float32)
    regfile = math.log2(1.0 + sm["registers"] * items / lanes)
    return np.concatenate([base, shp, base[:5] * shp[0], base[:5] * shp[1], base[:5] * shp[2], [regfile]]).astype(np.float32)


@dataclass
class KernelTuneResult:
    shapes: list                 # chosen shape per kernel
    us: np.ndarray               # time of each kernel in its chosen shape
    table: dict = field(default_factory=dict)  # shape -> per-kernel times (timed shapes only)
    seconds: float = 0.0
    timed: int = 0               # time_kernels passes

    @property
    def total_us(self) -> float:
        return float(self.us.sum())


def _apply_shapes(unit: native.Unit, shapes) -> None:
    for k, (i, l, t) in enumerate(shapes):
        unit.set_kernel_shape(k, i, l, t)


@dataclass(frozen=True)
class PerKernel:
    """A schedule kind run with the kernels' own launch shapes: tiles follow
    each kernel's shape (no fixed tile size)."""
    kind: str = "plain"
    executor: str = "interpreter"

    def apply(self, unit: native.Unit, math_mode: int = native.MATH_FAST, graph: int = 1) -> None:
        k, depth = KINDS[self.kind]
        unit.set_schedule(kind=k, math=math_mode, items_per_tile=0, use_graph=graph, fusion_depth=depth,
                          executor=EXECUTORS[self.executor])

    def __str__(self) -> str:
        return f"{self.kind} with per-kernel shapes ({self.executor})"


def tune_kernels(unit: native.Unit, flush=None, shapes=None, reps: int = 5,
                 executor: str = "interpreter") -> KernelTuneResult:
    """Exhaustive per-kernel tuning: every kernel timed in every shape."""
    if shapes is None:
        shapes = KERNEL_SHAPES if executor == "interpreter" else COMPILED_KERNEL_SHAPES
    t0 = time.perf_counter()
    PerKernel("plain", executor).apply(unit)
    nk = unit.num_kernels
    table = {}
    for sh in shapes:
        _apply_shapes(unit, [sh] * nk)
        try:
            unit.time_kernels(1, flush)
            table[sh] = unit.time_kernels(reps, flush)
        except RuntimeError:
            continue  # shape does not fit
    best = [min(table, key=lambda sh: table[sh][k]) for k in range(nk)]
    us = np.array([table[best[k]][k] for k in range(nk)])
    _apply_shapes(unit, best)
    return KernelTuneResult(best, us, table, time.perf_counter() - t0, len(table))


class KernelCostModel(CostModel):
    """MLP regression of log(kernel launch time in us) on kernel_features."""


def propose_kernel_shapes(model: KernelCostModel, unit: native.Unit, num_sets: int, k_top: int, summaries) -> list:
    """Top-k shapes per kernel by predicted time."""
    out = []
    for k in range(unit.num_kernels):
        X = np.stack([kernel_features(unit, k, num_sets, sh, summaries[k]) for sh in KERNEL_SHAPES])
        order = np.argsort(model.predict_us(X))
        out.append([KERNEL_SHAPES[i] for i in order[:k_top]])
    return out


def tune_kernels_with_model(unit: native.Unit, model: KernelCostModel, num_sets: int, flush=None, k_top: int = 2,
                            reps: int = 5) -> KernelTuneResult:
    """Times only each kernel's top-k proposed shapes (k passes of
    time_kernels, pass r putting every kernel in its r-th proposal)."""
    t0 = time.perf_counter()
    PerKernel("plain").apply(unit)
    summaries = [program_summary(unit, k) for k in range(unit.num_kernels)]
    props = propose_kernel_shapes(model, unit, num_sets, k_top, summaries)
    nk = unit.num_kernels
    best = [None] * nk
    us = np.full(nk, np.inf)
    passes = 0
    for r in range(k_top):
        _apply_shapes(unit, [p[r] for p in props])
        try:
            unit.time_kernels(1, flush)
            t = unit.time_kernels(reps, flush)
        except RuntimeError:
            continue
        passes += 1
        for k in range(nk):
            if t[k] < us[k]:
                us[k], best[k] = t[k], props[k][r]
    best = [b if b is not None else (1, 1, 128) for b in best]
    _apply_shapes(unit, best)
    return KernelTuneResult(best, us, {}, time.perf_counter() - t0, passes)
