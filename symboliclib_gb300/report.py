"""Measurements of the engine on the workloads beyond the headline benchmark.

    python -m symboliclib_gb300.report single --workload cloth --size 300 --sets 64
        plain per-call path (one value set, one launch per kernel, the
        reference's structure) against the batched, tuned engine on the same
        workload; nonzeros/s, algorithmic HBM GB/s and FP64 fraction.
    python -m symboliclib_gb300.report batch --count 64 --min-side 8 --max-side 48
        many cloth patterns of uneven size, 1-16 value sets each, evaluated by
        one CUDA-graph replay, against per-call plain evaluation of every set.
    python -m symboliclib_gb300.report learned --target neohookean --target-size 6
        the MLP cost model trained on tuner timings of other workloads, then
        used to pick the target's schedule: regret and tuning time against
        exhaustive search.
    python -m symboliclib_gb300.report kernels --target cloth --target-size 100 --sets 16
        per-kernel launch shapes: the kernel-level MLP (trained on other
        units' per-kernel timings) against exhaustive per-kernel tuning, and
        the tuned runs against the best unit-wide schedule.
    python -m symboliclib_gb300.report solve --size 300 --sets 8
        the cloth system matrix assembled by the engine, then solved on the
        device by the batched BiCGSTAB (the matrix is indefinite) or CG; SciPy's
        solver of the same method as CPU reference.
Each prints one JSON line.  Errors are measured against the workload's FP64
model evaluated in double (floor 1e-4 of the largest magnitude).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time
from pathlib import Path

import numpy as np

from . import native, tuner

PEAKS = Path(__file__).resolve().parent.parent / "MEASURED_PEAKS.json"


def hbm_peak():
    try:
        return float(json.loads(PEAKS.read_text())["hbm_gbs"])
    except Exception:
        return 6800.0


def rel_err(a, ref, floor_frac=1e-4):
    floor = floor_frac * np.max(np.abs(ref))
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor)))


def flush_buffer():
    import torch
    return torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2


def fp64_peak():
    v = C.c_double()
    native.check(native.symgb().symgb_measure_fp64_rate(C.byref(v)))
    return v.value


def single(args):
    t0 = time.perf_counter()
    w = native.Workload(args.workload, args.size, args.seed)
    front = time.perf_counter() - t0
    nnz = len(w.numeric)
    u = native.Unit.from_workload(w)
    stream = tuner.bind_stream(u)
    flush = flush_buffer()
    # plain per-call path: one value set, one launch per kernel
    for i, a in enumerate(w.inputs):
        u.set_arg(i, a)
    plain = tuner.Sched("plain", 1, 128, 1, 1, "compiled")
    plain.apply(u, graph=0)
    u.run()
    err_plain = rel_err(u.get_result(0), w.numeric)
    t_plain = tuner.time_schedule(u, plain, stream, flush, runs=args.steps) * 1e-6
    # batched value sets, tuned
    S = args.sets
    u.set_num_sets(S)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, np.tile(a, S))
    space = tuner.SPACE if args.full_space else [s for s in tuner.SPACE if s.tile == 1]
    tt = time.perf_counter()
    res = tuner.exhaustive(u, stream, flush, space=space, runs=max(3, args.steps // 2))
    t_batch = tuner.time_schedule(u, res.best, stream, flush, runs=args.steps) * 1e-6
    # per-kernel launch shapes (plain and levels schedules), kept if faster
    pk = tuner.tune_kernels(u, flush, reps=max(3, args.steps // 2))
    t_pk = {kind: tuner.time_schedule(u, tuner.PerKernel(kind), stream, flush, runs=args.steps) * 1e-6
            for kind in ("plain", "levels")}
    tune_s = time.perf_counter() - tt
    best_pk = min(t_pk, key=t_pk.get)
    chosen = f"{res.best}"
    if t_pk[best_pk] < t_batch:
        t_batch = t_pk[best_pk]
        chosen = f"{best_pk} with per-kernel shapes {[list(x) for x in pk.shapes]}"
        tuner.PerKernel(best_pk).apply(u)
    else:
        for k in range(u.num_kernels):
            u.set_kernel_shape(k)
        res.best.apply(u)
    u.run()
    out = u.get_result(0).reshape(S, -1)
    err_batch = max(rel_err(out[s], w.numeric) for s in (0, S - 1))
    st = u.stats()
    alg = u.algorithmic_bytes(S)
    peak = hbm_peak()
    fp = fp64_peak()
    flops = (st.flops + 10 * st.divs + 10 * st.sqrts) * S
    print(json.dumps({
        "workload": f"{args.workload} {args.size}", "output_nnz": nnz, "value_sets": S, "front_end_s": round(front, 1),
        "kernels": int(st.num_kernels), "levels": int(st.num_levels), "max_registers": int(st.max_registers),
        "plain": {"ms_per_execute": t_plain * 1e3, "nnz_per_s": nnz / t_plain, "max_rel_err": err_plain,
                  "hbm_gbs": u.algorithmic_bytes(1) / t_plain / 1e9},
        "batched": {"schedule": chosen, "unit_wide_best": str(res.best), "unit_wide_ms": res.best_us * 1e-3,
                    "per_kernel_plain_ms": t_pk["plain"] * 1e3, "per_kernel_levels_ms": t_pk["levels"] * 1e3,
                    "ms_per_execute": t_batch * 1e3, "nnz_per_s": nnz * S / t_batch,
                    "max_rel_err": err_batch, "algorithmic_bytes": alg, "hbm_gbs": alg / t_batch / 1e9,
                    "hbm_frac": alg / t_batch / 1e9 / peak, "fp64_tflops": flops / t_batch / 1e12,
                    "fp64_frac": flops / t_batch / fp, "tuning_s": round(tune_s, 1), "schedules_timed": res.timed + pk.timed},
        "speedup_batched_vs_plain": (nnz * S / t_batch) / (nnz / t_plain),
        "hbm_peak_gbs": peak, "fp64_peak_tflops": fp / 1e12}), flush=True)


# Schedules the batch's autotuning chooses from (compiled executor): the
# plain and levels shapes that win on cloth patterns from 16 x 16 to 300 x 300
# with 1 to 64 value sets.
BATCH_CANDIDATES = [tuner.Sched("plain", 4, 64, 1, 1, "compiled"), tuner.Sched("plain", 2, 128, 1, 1, "compiled"),
                    tuner.Sched("levels", 1, 128, 1, 1, "compiled"), tuner.Sched("levels", 4, 64, 1, 1, "compiled")]


def batch(args):
    import torch
    lib = native.symgb()
    rng = np.random.default_rng(args.seed)
    sides = np.exp(rng.uniform(math.log(args.min_side), math.log(args.max_side), args.count)).round().astype(int)
    sets = rng.integers(1, args.max_sets + 1, args.count)
    t0 = time.perf_counter()
    # one plan per distinct side (the pattern cache), built by several front
    # ends side by side, largest first
    from concurrent.futures import ThreadPoolExecutor
    distinct = sorted({int(x) for x in sides}, reverse=True)
    with ThreadPoolExecutor(max_workers=max(1, args.build_workers)) as ex:
        built = ex.map(lambda side: native.Workload("cloth", side, args.seed + side), distinct)
        cache = dict(zip(distinct, built))
    units, total_nnz, plain_s = [], 0, 0.0
    flush = flush_buffer()
    for k, (side, S) in enumerate(zip(sides, sets)):
        w = cache[int(side)]
        u = native.Unit.from_workload(w)
        units.append((u, int(S), w))
        total_nnz += len(w.numeric) * int(S)
    front = time.perf_counter() - t0
    # per-call plain evaluation of every value set (time of one set x S)
    stream = torch.cuda.Stream()
    plain_by_side = {}
    for u, S, w in units:
        native.check(lib.symgb_set_stream(u.handle, C.c_void_p(stream.cuda_stream)))
        key = w.size
        if key not in plain_by_side:
            for i, a in enumerate(w.inputs):
                u.set_arg(i, a)
            plain_by_side[key] = tuner.time_schedule(u, tuner.Sched("plain", 1, 128, 1, 1, "compiled"), stream, None,
                                                     runs=5) * 1e-6
        plain_s += plain_by_side[key] * S
    # batched: each unit with its sets; with --schedule tuned the autotuner
    # times BATCH_CANDIDATES on the first unit of every pattern (with that
    # unit's sets) and the pattern's other units take its choice; one graph
    chosen, t_tune = {}, time.perf_counter()
    for u, S, w in units:
        u.set_num_sets(S)
        for i, a in enumerate(w.inputs):
            u.set_arg(i, np.tile(a, S))
        if args.schedule == "tuned":
            if w.size not in chosen:
                ts = {c: tuner.time_schedule(u, c, stream, flush, runs=3) for c in BATCH_CANDIDATES}
                chosen[w.size] = min(ts, key=ts.get)
            chosen[w.size].apply(u, graph=0)
        else:
            tuner.Sched(args.schedule, args.items, args.tpb, 1, args.lanes, args.executor).apply(u, graph=0)
    tune_s = time.perf_counter() - t_tune
    handles = (C.c_void_p * len(units))(*[u.handle.value for u, _, _ in units])
    b = C.c_void_p()
    t_create = time.perf_counter()
    native.check(lib.symgb_batch_create(handles, len(units), args.streams, C.byref(b)))
    create_s = time.perf_counter() - t_create
    for _ in range(3):
        native.check(lib.symgb_batch_run(b))
    ts = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        native.check(lib.symgb_batch_run_async(b, C.c_void_p(stream.cuda_stream)))
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t_graph = float(np.median(ts))
    errs = []
    for u, S, w in units[:8]:
        out = u.get_result(0).reshape(S, -1)
        errs.append(rel_err(out[S - 1], w.numeric))
    launches = lib.symgb_batch_launch_count(b)
    lib.symgb_batch_destroy(b)
    print(json.dumps({
        "instances": int(args.count), "sides": [int(sides.min()), int(sides.max())], "distinct_patterns": len(cache),
        "value_sets_total": int(sets.sum()), "output_nnz_total": int(total_nnz), "front_end_s": round(front, 1),
        "graph": {"ms": t_graph * 1e3, "nnz_per_s": total_nnz / t_graph, "kernels": int(launches),
                  "streams": args.streams, "create_s": round(create_s, 1),
                  "schedule": ({str(c): sum(1 for v in chosen.values() if v == c) for c in BATCH_CANDIDATES}
                               if args.schedule == "tuned" else
                               f"{args.executor} {args.schedule} items {args.items} lanes {args.lanes} tpb {args.tpb}"),
                  "tuning_s": round(tune_s, 1)},
        "plain_per_call": {"ms": plain_s * 1e3, "nnz_per_s": total_nnz / plain_s},
        "speedup": plain_s / t_graph, "max_rel_err_sampled": max(errs)}), flush=True)


def learned(args):
    """Cost model trained on tuner timings of other workloads, applied to the target."""
    train = [("cotan", s, 1 + s) for s in (60, 120, 200)] + [("cloth", s, 2 + s) for s in (12, 20, 30)] + \
            [("ata", s, 3 + s) for s in (40, 70)] + [("random", n, 10 + k) for k, n in
                                                      enumerate([20000, 40000, 60000, 90000] * 5)]
    X, y = [], []
    t_collect = time.perf_counter()
    for spec in train:
        w = native.Workload(*spec)
        u = native.Unit.from_workload(w)
        for i, a in enumerate(w.inputs):
            u.set_arg(i, a)
        stream = tuner.bind_stream(u)
        for S in ((1, 8) if spec[0] in ("cloth", "cotan") else (1,)):
            u.set_num_sets(S)
            for i, a in enumerate(w.inputs):
                u.set_arg(i, np.tile(a, S))
            res = tuner.exhaustive(u, stream, runs=3)
            st = u.stats()
            for s, t in res.timings.items():
                X.append(tuner.features(st, S, s))
                y.append(t)
    t_collect = time.perf_counter() - t_collect
    model = tuner.CostModel(seed=args.seed)
    t_fit = time.perf_counter()
    loss = model.fit(np.stack(X), np.array(y), epochs=args.epochs)
    t_fit = time.perf_counter() - t_fit
    t_front = time.perf_counter()
    w = native.Workload(args.target, args.target_size, args.seed)
    t_front = time.perf_counter() - t_front
    u = native.Unit.from_workload(w)
    S = args.target_sets
    u.set_num_sets(S)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, np.tile(a, S))
    stream = tuner.bind_stream(u)
    flush = flush_buffer()
    # the learned proposal first, so its compiles are not served from the
    # exhaustive pass's module cache
    prop = tuner.tune_with_model(u, model, stream, flush, k=args.k, runs=5)
    full = tuner.exhaustive(u, stream, flush, runs=5)
    prop.best.apply(u)
    u.run()
    err = rel_err(u.get_result(0).reshape(S, -1)[0], w.numeric)
    print(json.dumps({
        "target": f"{args.target} {args.target_size}", "output_nnz": len(w.numeric), "value_sets": S,
        "front_end_s": round(t_front, 1), "max_rel_err_vs_fp64_model": err,
        "learned_nnz_per_s": len(w.numeric) * S / (full.timings.get(prop.best, prop.best_us) * 1e-6),
        "training_samples": len(y), "training_units": len(train), "collect_s": round(t_collect, 1),
        "fit_s": round(t_fit, 2), "fit_mse_log": loss,
        "exhaustive": {"best": str(full.best), "best_us": full.best_us, "timed": full.timed, "seconds": full.seconds},
        "learned": {"best": str(prop.best), "best_us": full.timings.get(prop.best, prop.best_us), "timed": prop.timed,
                    "seconds": prop.seconds},
        "regret": full.timings.get(prop.best, prop.best_us) / full.best_us - 1.0,
        "tuning_time_ratio": full.seconds / max(prop.seconds, 1e-9),
        "timings_ratio": full.timed / max(1, prop.timed)}), flush=True)


def kernels(args):
    """Per-kernel launch shapes: exhaustive per-kernel tuning against the
    learned per-kernel proposer (trained on other units' kernel timings), and
    the tuned plain / levels runs against the best unit-wide schedule."""
    flush = flush_buffer()
    train = [("cotan", s, 1 + s, S) for s in (60, 120, 200) for S in (1, 8)] + \
            [("cloth", s, 2 + s, S) for s in (12, 20, 30) for S in (1, 8)] + \
            [("ata", s, 3 + s, 1) for s in (40, 70)] + [("random", n, 10 + k, 1) for k, n in
                                                       enumerate([20000, 40000, 60000, 90000] * 3)]
    X, y = [], []
    t_collect = time.perf_counter()
    for name, size, seed, S in train:
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        u.set_num_sets(S)
        for i, a in enumerate(w.inputs):
            u.set_arg(i, np.tile(a, S))
        tuner.bind_stream(u)
        res = tuner.tune_kernels(u, flush, reps=3)
        sums = [tuner.program_summary(u, k) for k in range(u.num_kernels)]
        for sh, t in res.table.items():
            for k in range(u.num_kernels):
                if u.kernel_instances[k] and t[k] > 0:
                    X.append(tuner.kernel_features(u, k, S, sh, sums[k]))
                    y.append(t[k])
    t_collect = time.perf_counter() - t_collect
    model = tuner.KernelCostModel(seed=args.seed)
    loss = model.fit(np.stack(X), np.array(y), epochs=args.epochs)

    w = native.Workload(args.target, args.target_size, args.seed)
    S = args.sets
    u = native.Unit.from_workload(w)
    u.set_num_sets(S)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, np.tile(a, S))
    stream = tuner.bind_stream(u)
    unitwide = tuner.exhaustive(u, stream, flush, runs=5)
    full = tuner.tune_kernels(u, flush, reps=5)
    plain_tuned = tuner.time_schedule(u, tuner.PerKernel("plain"), stream, flush, runs=7)
    levels_tuned = tuner.time_schedule(u, tuner.PerKernel("levels"), stream, flush, runs=7)
    learned = tuner.tune_kernels_with_model(u, model, S, flush, k_top=args.k, reps=5)
    learned_total = float(sum(full.table[sh][k] for k, sh in enumerate(learned.shapes) if sh in full.table))
    u.run()
    err = rel_err(u.get_result(0).reshape(S, -1)[S - 1], w.numeric)
    print(json.dumps({
        "target": f"{args.target} {args.target_size}", "value_sets": S, "kernels": u.num_kernels,
        "training_samples": len(y), "training_units": len(train), "collect_s": round(t_collect, 1),
        "fit_mse_log": loss,
        "unit_wide_best": {"schedule": str(unitwide.best), "us": unitwide.best_us},
        "per_kernel_exhaustive": {"sum_of_kernels_us": full.total_us, "plain_run_us": plain_tuned,
                                  "levels_run_us": levels_tuned, "passes": full.timed, "seconds": full.seconds,
                                  "shapes": [list(s) for s in full.shapes]},
        "per_kernel_learned": {"sum_of_kernels_us": learned_total, "passes": learned.timed, "seconds": learned.seconds,
                               "k": args.k},
        "regret": learned_total / full.total_us - 1.0,
        "tuning_time_ratio": full.seconds / max(learned.seconds, 1e-9),
        "max_rel_err": err}), flush=True)


def solve(args):
    """Assembly of the cloth system matrix by the engine, then the batched
    conjugate-gradient solve on the device; SciPy's CG on the host for one
    system as the CPU reference."""
    import torch
    from scipy.sparse import csc_matrix
    from scipy.sparse.linalg import cg as scipy_cg
    w = native.Workload("cloth", args.size, args.seed)
    S = args.sets
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, items_per_thread=1, lanes_per_item=2,
                   threads_per_block=64)
    u.set_num_sets(S)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, np.tile(a, S))
    u.run()
    nnz = len(w.numeric)
    vals = torch.empty((S, nnz), dtype=torch.float64, device="cuda")
    native.check(native.symgb().symgb_get_result_sets_device(u.handle, C.c_void_p(vals.data_ptr()), 0))
    r, c, cp, ri = w.pattern()
    rng = np.random.default_rng(args.seed)
    b = torch.from_numpy(rng.standard_normal((S, r))).cuda()
    x = torch.empty_like(b)
    solver = native.SparseSolver(r, cp, ri, True, S)
    if args.block > 1:
        solver.set_block_preconditioner(args.block, r // args.block)
    method = native.SOLVER_BICGSTAB if args.method == "bicgstab" else native.SOLVER_CG
    solver.solve(vals, b, x, args.tol, 20, method)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it, res = solver.solve(vals, b, x, args.tol, args.max_iter, method)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    nnz_full = 2 * nnz - r
    # per iteration: BiCGSTAB two matrix products and ~26 vector passes, CG one and ~13
    mats, vecs = (2, 26) if method == native.SOLVER_BICGSTAB else (1, 13)
    per_iter_bytes = mats * (S * 8 * nnz_full + 4 * nnz_full + 8 * (r + 1)) + S * vecs * 8 * r
    # CPU reference: SciPy's solver of the same method, one system
    from scipy.sparse.linalg import bicgstab as scipy_bicgstab
    cpu_solver = scipy_bicgstab if method == native.SOLVER_BICGSTAB else scipy_cg
    L = csc_matrix((w.numeric, ri, cp), shape=(r, c))
    A = (L + L.T - csc_matrix((L.diagonal(), (np.arange(r), np.arange(r))), shape=(r, r))).tocsr()
    bh = b[0].cpu().numpy()
    t1 = time.perf_counter()
    it_cpu = [0]
    count = lambda _: it_cpu.__setitem__(0, it_cpu[0] + 1)
    try:
        xs, info = cpu_solver(A, bh, rtol=args.tol, maxiter=args.max_iter, callback=count)
    except TypeError:  # SciPy before 1.12 names the tolerance `tol`
        xs, info = cpu_solver(A, bh, tol=args.tol, maxiter=args.max_iter, callback=count)
    t_cpu = time.perf_counter() - t1
    resid = float(np.linalg.norm(A @ x[0].cpu().numpy() - bh) / np.linalg.norm(bh))
    print(json.dumps({
        "workload": f"cloth {args.size}", "preconditioner": f"block Jacobi {args.block}x{args.block}"
        if args.block > 1 else "scaled Jacobi", "unknowns": r, "nnz_lower": nnz, "nnz_full": nnz_full, "systems": S,
        "gpu": {"iterations": it, "max_rel_residual": res, "seconds": t, "us_per_iteration": t / max(1, it) * 1e6,
                "bytes_per_iteration": per_iter_bytes, "hbm_gbs": per_iter_bytes * it / t / 1e9,
                "hbm_frac": per_iter_bytes * it / t / 1e9 / hbm_peak(), "checked_residual_set0": resid},
        "method": args.method,
        "cpu_scipy_one_system": {"iterations": it_cpu[0], "seconds": t_cpu, "info": int(info)},
        "speedup_per_system": (t_cpu / max(1, it_cpu[0])) / (t / max(1, it) / S)}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("single")
    a.add_argument("--workload", default="cloth")
    a.add_argument("--size", type=int, default=300)
    a.add_argument("--sets", type=int, default=64)
    a.add_argument("--seed", type=int, default=2024)
    a.add_argument("--steps", type=int, default=10)
    a.add_argument("--full-space", action="store_true")
    b = sub.add_parser("batch")
    b.add_argument("--count", type=int, default=64)
    b.add_argument("--min-side", type=int, default=8)
    b.add_argument("--max-side", type=int, default=48)
    b.add_argument("--max-sets", type=int, default=16)
    b.add_argument("--streams", type=int, default=8)
    b.add_argument("--schedule", default="tuned", choices=["tuned"] + list(tuner.KINDS))
    b.add_argument("--items", type=int, default=1)
    b.add_argument("--lanes", type=int, default=1)
    b.add_argument("--executor", default="compiled", choices=["compiled", "interpreter"])
    b.add_argument("--tpb", type=int, default=64)
    b.add_argument("--seed", type=int, default=7)
    b.add_argument("--steps", type=int, default=10)
    b.add_argument("--build-workers", type=int, default=4, help="front ends building patterns side by side")
    c = sub.add_parser("learned")
    c.add_argument("--target", default="neohookean")
    c.add_argument("--target-size", type=int, default=6)
    c.add_argument("--target-sets", type=int, default=1)
    c.add_argument("--k", type=int, default=len(tuner.SPACE) // 15)
    c.add_argument("--epochs", type=int, default=4000)
    c.add_argument("--seed", type=int, default=5)
    d = sub.add_parser("kernels")
    d.add_argument("--target", default="cloth")
    d.add_argument("--target-size", type=int, default=100)
    d.add_argument("--sets", type=int, default=16)
    d.add_argument("--k", type=int, default=2)
    d.add_argument("--epochs", type=int, default=4000)
    d.add_argument("--seed", type=int, default=5)
    e = sub.add_parser("solve")
    e.add_argument("--size", type=int, default=300)
    e.add_argument("--sets", type=int, default=8)
    e.add_argument("--tol", type=float, default=1e-10)
    e.add_argument("--max-iter", type=int, default=5000)
    e.add_argument("--seed", type=int, default=3)
    e.add_argument("--method", default="bicgstab", choices=["cg", "bicgstab"])
    e.add_argument("--block", type=int, default=3, help="block-Jacobi block size (1: scaled Jacobi)")
    args = ap.parse_args()
    {"single": single, "batch": batch, "learned": learned, "kernels": kernels, "solve": solve}[args.cmd](args)


if __name__ == "__main__":
    main()
