"""Schedule autotuner and learned schedule proposer.

The schedule of a unit (launch structure, fusion depth, block size, work items
per thread, tile size) changes only speed, never values.  `exhaustive` times
every schedule in `SPACE` on the GPU and returns the fastest.  `CostModel` is
an MLP (the engine's FP32 kernels, native.MLP) that predicts the log run time
of a unit under a schedule from plan features; `propose` ranks all schedules
by predicted time and times only the top k, so tuning costs k timings instead
of len(SPACE).  The training data are timings the tuner itself collected."""
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


@dataclass(frozen=True)
class Sched:
    kind: str
    items: int
    tpb: int
    tile: int  # a tile is (tpb / lanes) * items * tile work items
    lanes: int = 1

    def apply(self, unit: native.Unit, math_mode: int = native.MATH_FAST, graph: int = 1) -> None:
        k, depth = KINDS[self.kind]
        unit.set_schedule(kind=k, math=math_mode, threads_per_block=self.tpb,
                          items_per_tile=self.tpb // self.lanes * self.items * self.tile, items_per_thread=self.items,
                          use_graph=graph, fusion_depth=depth, lanes_per_item=self.lanes)


# (items per thread, lanes per item): several items per thread for small
# register files, several lanes per item for large ones
SHAPES = ((1, 1), (2, 1), (4, 1), (1, 2), (1, 4))
SPACE = [Sched(k, i, t, f, l) for k, (i, l), t, f in itertools.product(KINDS, SHAPES, (64, 128, 256), (1, 4))]
DEFAULT = Sched("levels", 1, 128, 1)


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
    onehot = [1.0 if s.kind == k else 0.0 for k in KINDS]
    return np.array(onehot + [math.log2(s.lanes), math.log2(s.items), math.log2(s.tpb), math.log2(s.tile)], np.float32)


def features(stats: native.Stats, num_sets: int, s: Sched) -> np.ndarray:
    p = plan_features(stats, num_sets)
    q = schedule_features(s)
    # interactions: work per launch under this schedule
    # register file bytes per thread under this shape (occupancy)
    regfile = np.array([math.log2(1.0 + float(stats.max_registers) * s.items / s.lanes)], np.float32)
    return np.concatenate([p, q, p[:6] * q[-3] / 8.0, p[:6] * q[-2] / 8.0, p[:6] * q[-4] / 8.0, regfile])


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


def propose(model: CostModel, stats: native.Stats, num_sets: int, k: int = 3, space=SPACE) -> list[Sched]:
    X = np.stack([features(stats, num_sets, s) for s in space])
    order = np.argsort(model.predict_us(X))
    return [space[i] for i in order[:k]]


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
