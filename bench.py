"""Benchmark of ComputeUnit::execute() on the GB300 engine.

Workload (default): cotangent-Laplacian assembly (BuildCotan) on a 500 x 500
vertex grid (250,000 vertices, 498,002 triangles, 1,746,002 output nonzeros),
FP64, one value set - the plain-GPU-path configuration.  A step is one
execute(): every kernel of the plan over one batch of inputs.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl engine|reference]

Prints one JSON line (rank 0).  `value` is output nonzeros per second with the
inputs resident in HBM (device-timed, L2 flushed before every step); `e2e` is
the same metric through the C ABI with host buffers (pinned H2D copy of the
inputs, run, D2H copy of all outputs, every step).  `--impl reference` times
the reference's CPU ComputeUnit path (its generated-C-per-kernel structure,
restated by oracle/cpu_port.py) on all host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000, help="timed steps (default: a timed region of about a second, "
                                                                 "long enough for the clock samples)")
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="cotan")
    ap.add_argument("--size", type=int, default=500)
    ap.add_argument("--sets", type=int, default=1)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--schedule", default="levels", choices=["plain", "levels", "persistent"])
    ap.add_argument("--items", type=int, default=2, help="work items per thread (1, 2, 4)")
    ap.add_argument("--lanes", type=int, default=1, help="threads per work item (1, 2, 4, 8)")
    ap.add_argument("--tpb", type=int, default=64, help="threads per block")
    ap.add_argument("--math", default="fast", choices=["fast", "exact"])
    ap.add_argument("--executor", default="compiled", choices=["compiled", "interpreter"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-probe", action="store_true", help="skip the FP64 peak probe (e.g. under a profiler)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    return ap.parse_args()


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self._stop = index, [], threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.rows.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one step, summed
# over the step's evalKernel launches, from one ncu capture of that exact
# configuration on a GB300: (workload, size, sets, schedule, items, lanes,
# threads per block) -> bytes.  Configurations not captured report null.
MEASURED_TRAFFIC = {("cotan", 500, 1, "levels", 2, 1, 64): 82.45e6}


def peaks():
    try:
        p = json.loads(PEAKS_FILE.read_text())
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def rel_err(a, ref, floor_frac=1e-10):
    floor = floor_frac * np.max(np.abs(ref))
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor)))


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "engine" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config(args, w, extra=None):
    cfg = {"workload": f"{args.workload} {args.size}x{args.size} grid", "size": args.size,
           "output_nnz": int(len(w.numeric)), "value_sets": args.sets, "seed": args.seed}
    if extra:
        cfg.update(extra)
    return cfg


def run_reference(args):
    """CPU baseline arm: the reference's CPU path restated as generated C."""
    world, rank, _ = dist_init(args)
    if rank != 0:
        return
    from symboliclib_gb300 import build, native
    from oracle.cpu_port import CpuPort
    build.build()
    w = native.Workload(args.workload, args.size, args.seed)
    port = CpuPort(w.plan, w.index_data, w.out_index_data, w.const_data)
    nnz = len(w.numeric)
    times = []
    port.execute(w.inputs)
    for _ in range(args.warmup):
        port.execute(w.inputs)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        port.execute(w.inputs)
        times.append(time.perf_counter() - t0)
    err = rel_err(port.result(0), w.numeric, 1e-4)
    t = float(np.mean(times))
    v = nnz / t
    line = {"metric": "output nnz/s of execute()", "value": v, "unit": "nnz/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh)",
            "impl": "reference",
            "config": workload_config(args, w, {"path": "CPU ComputeUnit (generated C per kernel, OpenMP, "
                                                       "-O3 -ffast-math)", "max_rel_err_vs_fp64_model": err}),
            "cpu_baseline": {"value": v, "unit": "nnz/s", "cores": port.threads, "kind": "port",
                             "sample": f"{args.steps} executes of the full workload"},
            "e2e": {"value": v, "unit": "nnz/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_engine(args):
    world, rank, local = dist_init(args)
    import torch
    torch.cuda.set_device(local)
    from symboliclib_gb300 import build, native
    build.build()

    kinds = {"plain": native.SCHEDULE_PLAIN, "levels": native.SCHEDULE_LEVELS,
             "persistent": native.SCHEDULE_PERSISTENT}
    t0 = time.perf_counter()
    w = native.Workload(args.workload, args.size, args.seed)
    front_s = time.perf_counter() - t0
    S = args.sets
    nnz = len(w.numeric)
    u = native.Unit.from_workload(w)
    stream = torch.cuda.Stream()
    native.check(native.symgb().symgb_set_stream(u.handle, C.c_void_p(stream.cuda_stream)))
    execs = {"compiled": native.EXEC_COMPILED, "interpreter": native.EXEC_INTERPRETER}
    u.set_schedule(kind=kinds[args.schedule], math=native.MATH_FAST if args.math == "fast" else native.MATH_EXACT,
                   threads_per_block=args.tpb, items_per_thread=args.items, lanes_per_item=args.lanes,
                   executor=execs[args.executor])
    u.set_num_sets(S)
    compile_s = u.prepare()
    inputs = [np.tile(a, S) for a in w.inputs]
    for i, a in enumerate(inputs):
        u.set_arg(i, a)
    u.run()
    out = u.get_result(0).reshape(S, -1)
    err = max(rel_err(out[s], w.numeric, 1e-4) for s in range(S))
    lib = native.symgb()

    # device-resident timing: L2 flushed (256 MiB write) before each step
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            native.check(lib.symgb_run_async(u.handle))
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        launches = 0
        with ClockSampler(local) as clk:
            for k in range(args.steps):
                flush.fill_(float(k))
                ev[k][0].record(stream)
                native.check(lib.symgb_run_async(u.handle))
                ev[k][1].record(stream)
                launches += u.last_launch_count()
            torch.cuda.synchronize()
        barrier(world)
    native.check(lib.symgb_synchronize(u.handle))
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_step = max_over_ranks(world, float(np.mean(step_ms)) * 1e-3)
    value = world * nnz * S / t_step

    # end-to-end through the C ABI with pinned host buffers
    pinned_in = [torch.from_numpy(a).pin_memory() for a in inputs]
    pinned_out = torch.empty(nnz * S, dtype=torch.float64).pin_memory()
    for _ in range(2):
        for i, a in enumerate(pinned_in):
            native.check(lib.symgb_set_arg_sets(u.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run(u.handle))
        native.check(lib.symgb_get_result_sets(u.handle, C.c_void_p(pinned_out.data_ptr()), 0))
    barrier(world)
    e2e_steps = max(3, args.steps // 2)
    # (a) one execute at a time: set_arg, run, get_result, each waiting
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for i, a in enumerate(pinned_in):
            native.check(lib.symgb_set_arg_sets(u.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run(u.handle))
        native.check(lib.symgb_get_result_sets(u.handle, C.c_void_p(pinned_out.data_ptr()), 0))
    t_seq = max_over_ranks(world, (time.perf_counter() - t0) / e2e_steps)
    e2e_err = rel_err(pinned_out.numpy().reshape(S, -1)[0], w.numeric, 1e-4)
    # (b) pipelined: two units of the plan on two streams take alternate
    # steps; every step still copies its inputs in, evaluates and gathers its
    # results into pinned host memory (the ABI's async calls), in order on its
    # unit's stream, so one step's transfers overlap the other's evaluation.
    u2 = native.Unit.from_workload(w)
    u2.set_schedule(kind=kinds[args.schedule], math=native.MATH_FAST if args.math == "fast" else native.MATH_EXACT,
                    threads_per_block=args.tpb, items_per_thread=args.items, lanes_per_item=args.lanes,
                    executor=execs[args.executor])
    u2.set_num_sets(S)
    stream2 = torch.cuda.Stream()
    native.check(lib.symgb_set_stream(u2.handle, C.c_void_p(stream2.cuda_stream)))
    pipe = [(u, pinned_in, pinned_out),
            (u2, [torch.from_numpy(a).pin_memory() for a in inputs], torch.empty(nnz * S, dtype=torch.float64).pin_memory())]

    def pipelined_step(k):
        uu, pin_i, pin_o = pipe[k % 2]
        for i, a in enumerate(pin_i):
            native.check(lib.symgb_set_arg_sets_async(uu.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run_async(uu.handle))
        native.check(lib.symgb_get_result_sets_async(uu.handle, C.c_void_p(pin_o.data_ptr()), 0))

    for k in range(4):
        pipelined_step(k)
    for uu, _, _ in pipe:
        native.check(lib.symgb_synchronize(uu.handle))
    barrier(world)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        pipelined_step(k)
    for uu, _, _ in pipe:
        native.check(lib.symgb_synchronize(uu.handle))
    t_e2e = max_over_ranks(world, (time.perf_counter() - t0) / e2e_steps)
    barrier(world)
    e2e_err = max(e2e_err, rel_err(pipe[1][2].numpy().reshape(S, -1)[0], w.numeric, 1e-4))

    # plain schedule (the reference's per-kernel launch structure) for comparison
    u.set_schedule(kind=native.SCHEDULE_PLAIN, math=native.MATH_FAST, executor=execs[args.executor])
    u.prepare()
    with torch.cuda.stream(stream):
        for _ in range(3):
            native.check(lib.symgb_run_async(u.handle))
        pl = []
        for k in range(max(5, args.steps // 2)):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            native.check(lib.symgb_run_async(u.handle))
            b.record(stream)
            pl.append((a, b))
        torch.cuda.synchronize()
    t_plain = float(np.mean([a.elapsed_time(b) for a, b in pl])) * 1e-3

    stats = u.stats()
    alg_bytes = u.algorithmic_bytes(S)
    peak, peak_kind = peaks()
    achieved = alg_bytes / t_step / 1e9
    fp64 = C.c_double(1.25e12)  # nominal GB300 FP64 rate when the probe is skipped
    if not args.no_fp64_probe:
        native.check(lib.symgb_measure_fp64_rate(C.byref(fp64)))
    flops = (stats.flops + 10 * stats.divs + 10 * stats.sqrts) * S

    if rank != 0:
        return
    line = {"metric": "output nnz/s of execute()", "value": value, "unit": "nnz/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh)",
            "config": workload_config(args, w, {
                "schedule": args.schedule, "executor": args.executor, "compile_s": round(compile_s, 2),
                "items_per_thread": args.items, "lanes_per_item": args.lanes,
                "threads_per_block": args.tpb, "math": args.math, "l2": "flushed before every step (256 MiB write)",
                "front_end_s": round(front_s, 2), "kernels": int(stats.num_kernels), "levels": int(stats.num_levels),
                "max_rel_err_vs_fp64_model": err, "plain_schedule_ms_per_step": t_plain * 1e3,
                "plain_schedule_nnz_per_s": world * nnz * S / t_plain,
                "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}),
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": MEASURED_TRAFFIC.get((args.workload, args.size, S, args.schedule, args.items,
                                                          args.lanes, args.tpb)),
                         "traffic_unit": "bytes per step (ncu capture)",
                         "algorithmic_bytes_per_step": alg_bytes},
            "fp64": {"flops_per_step": flops, "achieved_tflops": flops / t_step / 1e12,
                     "peak_tflops": fp64.value / 1e12, "peak_source": "nominal" if args.no_fp64_probe else "measured",
                     "frac": flops / t_step / fp64.value},
            "e2e": {"value": world * nnz * S / t_e2e, "unit": "nnz/s", "ms_per_step": t_e2e * 1e3,
                    "h2d_bytes_per_step": int(sum(a.nbytes for a in inputs)), "d2h_bytes_per_step": int(nnz * S * 8),
                    "max_rel_err_vs_fp64_model": e2e_err,
                    "mode": "two units on two streams take alternate steps (async set_arg / run / get_result: "
                            "results gathered on the device and copied to pinned memory on the unit's copy "
                            "stream); every step copies its inputs in and its results out; no L2 flush",
                    "one_at_a_time": {"value": world * nnz * S / t_seq, "ms_per_step": t_seq * 1e3}},
            "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        from oracle.cpu_port import CpuPort
        port = CpuPort(w.plan, w.index_data, w.out_index_data, w.const_data)
        t_cpu, runs = port.time_execute(w.inputs, budget_s=args.cpu_budget)
        line["cpu_baseline"] = {"value": nnz / t_cpu, "unit": "nnz/s", "cores": port.threads, "kind": "port",
                                "sample": f"median of {runs} full executes (1 value set)"}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
