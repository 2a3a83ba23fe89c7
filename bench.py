"""Benchmark of ComputeUnit::execute() on the GB300 engine.

Workload (default): the Baraff-Witkin cloth Hessian A = M - h (D + h K) of a
300 x 300 vertex grid (90,000 vertices, 178,802 triangles, 3,762,024 output
nonzeros of the lower triangle), FP64, 64 value sets (time steps) of one
sparsity pattern evaluated per execute, schedule tuned on the spot by the
engine's own autotuner over a small space.  A step is one execute(): every
kernel of the plan over all 64 value sets.  `--workload cotan --size 500
--sets 1` gives the cotangent-Laplacian plain-GPU-path configuration.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl engine|reference]

Prints one JSON line (rank 0).  `value` is output nonzeros per second (all
value sets) with the inputs resident in HBM, device-timed with CUDA events on
the unit's stream; `e2e` is the same metric through the C ABI with host
buffers (page-locked input copies in and result copies out every step, two
units pipelined).  `config.plain_per_call` is the plain per-call GPU path:
one value set per execute, one launch per kernel.  `--impl reference` times
the reference's own CPU ComputeUnit: the C++ its ComputeUnit generated for
Device(VecWidth(4)) (kept by oracle/ref_generate.sh), compiled on this host
with NUMTHREADS = the host's cores; beside it the reference's generated CUDA
(its plain GPU path) is timed on the GPU.  Where that generated code was not
kept (cloth 300 x 300: the reference's front end needs more host memory than
the machine that made the others had), the CPU leg is oracle/cpu_port.py, a
generated-C restatement of the same structure (`kind: "port"`).
"""
from __future__ import annotations

import argparse
import atexit
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
METRIC = "output nnz/s of execute()"
# Relative error per nonzero against the FP64 numeric model: entries below a
# floor (a fraction of the container's largest magnitude) are compared against
# the floor.  The assembled matrices (cotangent Laplacian, cloth and
# Neo-Hookean Hessians) have entries that are sums of terms up to 1e4 times
# the result, where any two evaluation orders differ by more than 1e-12
# relative (the reference's own order is 4.8e-11 from the FP64 model on
# cotan 500x500 entries below 1e-6 of the largest), so their floor is 1e-4,
# as for A^T A + A, whose smallest entries are sums that cancel; 1e-10
# elsewhere (as in tests/).
TOL = 1e-12
FLOOR = {"cloth": 1e-4, "neohookean": 1e-4, "cotan": 1e-4, "ata": 1e-4}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="cloth")
    ap.add_argument("--size", type=int, default=300)
    ap.add_argument("--sets", type=int, default=64)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--schedule", default="tuned", choices=["tuned", "plain", "levels", "persistent"])
    ap.add_argument("--items", type=int, default=1, help="work items per thread (1, 2, 4)")
    ap.add_argument("--lanes", type=int, default=1, help="threads per work item (interpreter: 1, 2, 4, 8)")
    ap.add_argument("--tpb", type=int, default=128, help="threads per block")
    ap.add_argument("--min-blocks", type=int, default=0,
                    help="compiled executor: minimum resident CTAs per SM the kernels are compiled for (0: compiler)")
    ap.add_argument("--math", default="fast", choices=["fast", "exact"])
    ap.add_argument("--executor", default="compiled", choices=["compiled", "interpreter"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-probe", action="store_true", help="skip the FP64 peak probe (e.g. under a profiler)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end loops (e.g. under a profiler)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    return ap.parse_args()


class ClockSampler:
    """Clocks and throttle reasons every 200 ms from one long-running
    `nvidia-smi -lms 200` started before the workload is built (forking a
    process that holds a large plan can stall the launching thread for a
    long time; one child started early forks once, while the process is
    small).  mark_start / mark_stop bound the timed region; the summary uses
    the samples taken inside it."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.rows = []  # (time, fields)
        self.window = (None, None)
        try:
            self._p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.FIELDS}",
                                        "--format=csv,noheader,nounits", "-lms", "200"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._p = None
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        atexit.register(self.close)

    def _read(self):
        if self._p is None:
            return
        for line in self._p.stdout:
            self.rows.append((time.time(), [v.strip() for v in line.strip().split(",")]))

    def mark_start(self):
        self.window = (time.time(), None)

    def mark_stop(self):
        time.sleep(0.25)  # one more sample after the region
        self.window = (self.window[0], time.time())

    def close(self):
        if self._p is not None and self._p.poll() is None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()

    def summary(self):
        t0, t1 = self.window
        rows = [r for t, r in self.rows if t0 is not None and t1 is not None and t0 <= t <= t1]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# Per-step DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum over the
# step's launches) and FP64 pipe utilisation per launch from ncu captures of
# the compiled executor on a GB300, summarised (with their commands) in
# profiles/.  Keyed by (workload, size, value sets, schedule kind, threads per
# block, items per thread, minimum CTAs per SM); configurations not captured
# report null.
MEASURED = {
    ("cotan", 500, 1, "levels", 128, 1, 0): {"traffic": 81.77e6, "fp64_pipe_busy": [0.819, 0.851, 0.411],
                                             "profile": "profiles/symgb_cotan500_levels.md"},
    # full size, single-pass captures: symgb_k1 (the face-block template)
    # 389.07 MB read + 8.18 GB written per launch; the step's 18 kernels
    # 18.707 GB; k1's FP64 pipe share from the full section set on cloth
    # 100 x 100 x 16 sets
    ("cloth", 300, 64, "plain", 64, 4, 0): {"kernel_traffic": 8.569e9, "kernel_fp64_pipe_busy": 0.853,
                                            "traffic": 18.707e9,
                                            "profile": "profiles/symgb_cloth100_k1.md, "
                                                       "profiles/traffic_cloth300x64_plain.md"},
}


def peaks():
    try:
        p = json.loads(PEAKS_FILE.read_text())
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def rel_err(a, ref, floor_frac):
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


def workload_name(args):
    grid = "x".join([str(args.size)] * (3 if args.workload == "neohookean" else 2))
    return f"{args.workload} {grid}"


# ------------------------------------------------------------------ reference arm

def reference_cpu(args, budget_s: float, max_steps: int):
    """The reference CPU ComputeUnit on this host's cores: its generated C++
    (VecWidth(4), NUMTHREADS = cores) when oracle/ref_generate.sh kept it,
    else the CPU port of its structure (oracle/cpu_port.py).  Returns
    (ms per execute of one value set, cores, kind, sample, path)."""
    from oracle import ref_paths
    if ref_paths.available(args.workload, args.size, "cpu"):
        r = ref_paths.cpu_execute(args.workload, args.size, budget_s, max_steps)
        return (r["execute_ms"], r["threads"], "reference",
                f"median of {r['steps']} execute() calls (setArg + run, one value set each)",
                "the reference's generated cpuCode.cpp, Device(VecWidth(4)), -DNUMTHREADS=cores, built by "
                "the reference's clang++ command line mapped onto g++ (oracle/ref_clangxx.sh)")
    from symboliclib_gb300 import build, native
    from oracle.cpu_port import CpuPort
    build.build()
    w = native.Workload(args.workload, args.size, args.seed)
    port = CpuPort(w.plan, w.index_data, w.out_index_data, w.const_data)
    t, runs = port.time_execute(w.inputs, budget_s=budget_s)
    return (t * 1e3, port.threads, "port", f"median of {runs} execute() calls (one value set each)",
            "CPU port of the reference's generated-C structure (the reference's generated code was not "
            "kept for this workload)")


def reference_gpu(args):
    """The reference's plain GPU path (its generated CUDA) for one value set,
    three builds; None when its generated code was not kept."""
    from oracle import ref_paths
    if not ref_paths.available(args.workload, args.size, "cuda"):
        return None
    res = ref_paths.gpu_paths(args.workload, args.size, warmup=5, steps=max(20, min(200, args.steps)))
    out = {"note": "one value set per run(), one launch per kernel; median run() time with CUDA events on the "
                   "library's stream, L2 cleared before every run"}
    for k, label in (("ref_default", "reference nvcc command (compute_75 PTX, driver JIT)"),
                     ("ref_sm103a", "-arch=sm_103a"), ("ref_exact", "-arch=sm_103a --fmad=false")):
        out[k] = {"build": label, "ms_per_execute": res[k]["run_event_ms"], "run_host_ms": res[k]["run_ms"],
                  "execute_host_ms": res[k]["execute_ms"],
                  "nnz_per_s": res[k]["outputs"] / (res[k]["run_event_ms"] * 1e-3)}
    return out


def run_reference(args):
    world, rank, _ = dist_init(args)
    if rank != 0:
        return
    ms, cores, kind, sample, path = reference_cpu(args, budget_s=max(10.0, args.cpu_budget * 2), max_steps=args.steps)
    from oracle import ref_paths
    d = ref_paths.gen_dir(args.workload, args.size, "cpu")
    if (d / "outIndexData").exists():
        nnz = (d / "outIndexData").stat().st_size // 4
    else:
        from symboliclib_gb300 import native
        nnz = len(native.Workload(args.workload, args.size, args.seed).numeric)
    v = nnz / (ms * 1e-3)
    line = {"metric": METRIC, "value": v, "unit": "nnz/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh)", "impl": "reference",
            "config": {"workload": workload_name(args), "size": args.size, "output_nnz": nnz, "seed": args.seed,
                       "value_sets": 1, "path": path},
            "cpu_baseline": {"value": v, "unit": "nnz/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": "nnz/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    try:
        g = reference_gpu(args)
        if g is not None:
            line["ref_gpu"] = g
    except Exception as e:  # the CPU arm stands on its own
        line["ref_gpu"] = {"unavailable": str(e)[-300:]}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ engine arm

# Candidates of the on-the-spot tuning (compiled executor): kind, threads per
# block, items per thread.
TUNE_SPACE = [("plain", 64, 4, 0), ("plain", 128, 2, 0), ("plain", 128, 4, 0), ("levels", 64, 4, 0),
              ("levels", 128, 1, 0), ("levels", 128, 2, 0), ("levels", 256, 1, 0), ("persistent", 128, 4, 0)]


def fp64_instructions(u, tuner, math):
    """FP64-pipe instructions of one value set, counted from the kernels'
    programs: one per add, subtract, multiply and FMA; the fast division
    (two refinement FMAs, a product and two correction FMAs after the
    approximate reciprocal) 5, the fast square root 6, the fast reciprocal 4
    (exact mode's IEEE division and square root take more)."""
    total = 0
    for k in range(u.num_kernels):
        sm = tuner.program_summary(u, k, math)
        per = sm["add"] + sm["sub"] + sm["mul"] + sm["fma"] + 5 * sm["div"] + 6 * sm["sqrt"] + 4 * sm["rec"]
        total += per * u.kernel_instances[k]
    return total


def main_engine(args):
    world, rank, local = dist_init(args)
    clk = ClockSampler(local)
    import torch
    torch.cuda.set_device(local)
    from symboliclib_gb300 import build, native
    build.build()
    lib = native.symgb()
    kinds = {"plain": native.SCHEDULE_PLAIN, "levels": native.SCHEDULE_LEVELS,
             "persistent": native.SCHEDULE_PERSISTENT}
    execs = {"compiled": native.EXEC_COMPILED, "interpreter": native.EXEC_INTERPRETER}
    math = native.MATH_FAST if args.math == "fast" else native.MATH_EXACT
    floor = FLOOR.get(args.workload, 1e-10)

    t0 = time.perf_counter()
    w = native.Workload(args.workload, args.size, args.seed)
    front_s = time.perf_counter() - t0
    S = args.sets
    nnz = len(w.numeric)
    inputs = [np.tile(a, S) for a in w.inputs]  # S value sets (the same state in each)

    def make_unit():
        u = native.Unit.from_workload(w)
        st = torch.cuda.Stream()
        native.check(lib.symgb_set_stream(u.handle, C.c_void_p(st.cuda_stream)))
        u.set_num_sets(S)
        return u, st

    def apply(u, kind, tpb, items, minb):
        u.set_schedule(kind=kinds[kind], math=math, threads_per_block=tpb, items_per_thread=items,
                       lanes_per_item=args.lanes, executor=execs[args.executor], blocks_per_sm=minb)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def time_runs(u, st, runs, warmup=2):
        with torch.cuda.stream(st):
            for _ in range(warmup):
                native.check(lib.symgb_run_async(u.handle))
            evs = []
            for k in range(runs):
                flush.fill_(float(k))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                native.check(lib.symgb_run_async(u.handle))
                b.record(st)
                evs.append((a, b))
            torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    u, stream = make_unit()
    for i, a in enumerate(inputs):
        u.set_arg(i, a)
    # schedule: tuned on the spot (median of 3 runs per candidate) or given
    tuning = None
    t_tune = time.perf_counter()
    compile_s = 0.0
    if args.schedule == "tuned":
        timings = {}
        for cand in TUNE_SPACE:
            apply(u, *cand)
            compile_s += u.prepare()
            timings[cand] = float(np.median(time_runs(u, stream, 3)))
        best = min(timings, key=timings.get)
        tuning = {"candidates_ms": {f"{k} tpb{t} items{i}" + (f" minblocks{m}" if m else ""): round(v, 4)
                                    for (k, t, i, m), v in timings.items()},
                  "seconds": round(time.perf_counter() - t_tune, 1)}
        kind, tpb, items, minb = best
    else:
        kind, tpb, items, minb = args.schedule, args.tpb, args.items, args.min_blocks
    apply(u, kind, tpb, items, minb)
    compile_s += u.prepare()
    u.run()
    out = u.get_result(0).reshape(S, -1)
    err = max(rel_err(out[s], w.numeric, floor) for s in (0, S - 1))

    # device-resident timing: L2 cleared (256 MiB write) before every step
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            native.check(lib.symgb_run_async(u.handle))
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        clk.mark_start()
        launches = 0
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            native.check(lib.symgb_run_async(u.handle))
            ev[k][1].record(stream)
            launches += u.last_launch_count()
        torch.cuda.synchronize()
        barrier(world)
    clk.mark_stop()
    native.check(lib.symgb_synchronize(u.handle))
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_step = max_over_ranks(world, float(np.mean(step_ms)) * 1e-3)
    value = world * nnz * S / t_step

    # dominant kernel: every kernel timed with CUDA events on the unit's
    # stream over as many steps as the timed region (plain launches of the
    # chosen shape, L2 cleared before every step)
    us_k = u.time_kernels(reps=args.steps, flush=flush)
    kd = int(np.argmax(us_k))

    # plain per-call path: one value set per execute, one launch per kernel
    up = native.Unit.from_workload(w)
    stp = torch.cuda.Stream()
    native.check(lib.symgb_set_stream(up.handle, C.c_void_p(stp.cuda_stream)))
    for i, a in enumerate(w.inputs):
        up.set_arg(i, a)
    up.set_schedule(kind=native.SCHEDULE_PLAIN, math=math, threads_per_block=128, executor=native.EXEC_COMPILED)
    up.prepare()
    up.run()
    err_plain = rel_err(up.get_result(0), w.numeric, floor)
    t_plain = float(np.median(time_runs(up, stp, max(10, min(200, args.steps))))) * 1e-3
    up.close()
    del up

    # end to end through the C ABI with page-locked host buffers
    e2e = None
    if not args.no_e2e:
        e2e = end_to_end(args, w, u, make_unit, apply, (kind, tpb, items, minb), inputs, nnz, S, floor, world, lib,
                         native, torch)

    stats = u.stats()
    alg_bytes = u.algorithmic_bytes(S)
    peak, peak_kind = peaks()
    achieved = alg_bytes / t_step / 1e9
    fp64 = C.c_double(1.25e12)  # nominal GB300 FP64 rate when the probe is skipped
    if not args.no_fp64_probe:
        native.check(lib.symgb_measure_fp64_rate(C.byref(fp64)))
    flops_w = (stats.flops + 10 * stats.divs + 10 * stats.sqrts) * S
    from symboliclib_gb300 import tuner
    fp64_instr = fp64_instructions(u, tuner, math) * S
    meas = MEASURED.get((args.workload, args.size, S, kind, tpb, items, minb), {})
    # the dominant kernel's algorithmic bytes per launch: every gathered value
    # and every result once per value set, its index and constant rows once
    kdesc = w.plan.contents.kernels[kd]
    ksum = tuner.program_summary(u, kd, math)
    n_k = int(kdesc.num_instances)
    k_bytes = S * 8 * n_k * (ksum["ldx"] + ksum["st"]) + 8 * n_k * ksum["ldc"] + 4 * n_k * int(kdesc.num_index_rows)
    k_fp64 = (ksum["add"] + ksum["sub"] + ksum["mul"] + ksum["fma"] + 5 * ksum["div"] + 6 * ksum["sqrt"] +
              4 * ksum["rec"]) * n_k * S
    t_k = us_k[kd] * 1e-6

    if rank != 0:
        return
    cfg = {"workload": workload_name(args), "size": args.size, "output_nnz": nnz, "value_sets": S,
           "seed": args.seed, "inputs": "the seeded state, the same in every value set",
           "schedule": kind, "executor": args.executor, "threads_per_block": tpb, "items_per_thread": items,
           "min_blocks_per_sm": minb,
           "math": args.math, "tuning": tuning, "compile_s": round(compile_s, 2),
           "l2": "cleared before every step (256 MiB write)",
           "front_end_s": round(front_s, 1), "model_s": round(w.model_seconds, 1),
           "kernels": int(stats.num_kernels), "levels": int(stats.num_levels),
           "max_rel_err_vs_fp64_model": err, "tolerance": {"rel": TOL, "floor_frac": floor},
           "plain_per_call": {"ms_per_execute": t_plain * 1e3, "nnz_per_s": world * nnz / t_plain,
                              "max_rel_err_vs_fp64_model": err_plain,
                              "path": "compiled executor, plain schedule (one launch per kernel, the reference's "
                                      "run() structure), one value set per execute"},
           "speedup_vs_plain_per_call": value / (world * nnz / t_plain),
           "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}
    line = {"metric": METRIC, "value": value, "unit": "nnz/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh)", "config": cfg,
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": f"symgb_k{kd}", "achieved": k_bytes / t_k / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": k_bytes / t_k / 1e9 / peak, "peak_source": peak_kind,
                         "traffic": meas.get("kernel_traffic"),
                         "traffic_unit": "DRAM bytes per launch of the kernel (ncu capture)",
                         "algorithmic_bytes_per_launch": k_bytes, "ms_per_launch": t_k * 1e3,
                         "launches_per_step": 1, "share_of_step": t_k / t_step,
                         "fp64_instructions_per_launch": k_fp64,
                         "fp64_pipe_frac": k_fp64 / t_k / (fp64.value / 2),
                         "fp64_pipe_busy_ncu": meas.get("kernel_fp64_pipe_busy"),
                         "timing": "CUDA events around every kernel on the unit's stream, plain launches of the "
                                   "chosen shape, as many steps as the timed region, L2 cleared before each",
                         "bytes_note": "every gathered value and every result once per value set, index and "
                                       "constant rows once"},
            "roofline_step": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                              "frac": achieved / peak, "peak_source": peak_kind,
                              "traffic": meas.get("traffic"), "traffic_unit": "DRAM bytes per step (ncu capture)",
                              "algorithmic_bytes_per_step": alg_bytes},
            "fp64": {"flops_per_step_weighted": flops_w, "achieved_tflops": flops_w / t_step / 1e12,
                     "peak_tflops": fp64.value / 1e12,
                     "peak_source": "nominal" if args.no_fp64_probe else "measured",
                     "frac_flop_weighted": flops_w / t_step / fp64.value,
                     "weighting": "add/mul 1, FMA 2, division and square root 10 flops",
                     "instructions_per_step": fp64_instr,
                     "pipe_frac_instructions": fp64_instr / t_step / (fp64.value / 2),
                     "pipe_frac_note": "FP64 instructions the programs issue per step (fast division 5, square "
                                       "root 6) / step time / the measured FMA rate",
                     "pipe_busy_ncu": meas.get("fp64_pipe_busy"), "profile": meas.get("profile")},
            "clocks": clk.summary()}
    clk.close()
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu_baseline:
        try:
            ms, cores, kind_c, sample, path = reference_cpu(args, args.cpu_budget, max_steps=200)
            line["cpu_baseline"] = {"value": nnz / (ms * 1e-3), "unit": "nnz/s", "cores": cores, "kind": kind_c,
                                    "sample": sample, "path": path}
        except Exception as e:
            line["cpu_baseline"] = {"unavailable": str(e)[-300:]}
    print(json.dumps(line), flush=True)


def end_to_end(args, w, u, make_unit, apply, sched, inputs, nnz, S, floor, world, lib, native, torch):
    """Every step copies its inputs from page-locked host memory, evaluates and
    copies all results back (the ABI's async calls).  Two units of the plan on
    two streams take alternate steps, so one step's transfers overlap the
    other's evaluation; `one_at_a_time` waits for every call."""
    pinned_in = [torch.from_numpy(a).pin_memory() for a in inputs]
    pinned_out = torch.empty(nnz * S, dtype=torch.float64).pin_memory()
    steps = max(3, min(args.steps, 50))
    for _ in range(2):
        for i, a in enumerate(pinned_in):
            native.check(lib.symgb_set_arg_sets(u.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run(u.handle))
        native.check(lib.symgb_get_result_sets(u.handle, C.c_void_p(pinned_out.data_ptr()), 0))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        for i, a in enumerate(pinned_in):
            native.check(lib.symgb_set_arg_sets(u.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run(u.handle))
        native.check(lib.symgb_get_result_sets(u.handle, C.c_void_p(pinned_out.data_ptr()), 0))
    t_seq = max_over_ranks(world, (time.perf_counter() - t0) / steps)
    got = pinned_out.numpy().reshape(S, -1)
    err = max(rel_err(got[s], w.numeric, floor) for s in (0, S - 1))
    u2, _ = make_unit()
    apply(u2, *sched)
    u2.prepare()
    pipe = [(u, pinned_in, pinned_out),
            (u2, [torch.from_numpy(a).pin_memory() for a in inputs],
             torch.empty(nnz * S, dtype=torch.float64).pin_memory())]

    def step(k):
        uu, pin_i, pin_o = pipe[k % 2]
        for i, a in enumerate(pin_i):
            native.check(lib.symgb_set_arg_sets_async(uu.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run_async(uu.handle))
        native.check(lib.symgb_get_result_sets_async(uu.handle, C.c_void_p(pin_o.data_ptr()), 0))

    # the result copy on 1 or 4 copy streams (several copy engines), the
    # faster one reported
    by_streams = {}
    for cs in (1, 4):
        for uu, _, _ in pipe:
            uu.set_copy_streams(cs)
        for k in range(4):
            step(k)
        for uu, _, _ in pipe:
            native.check(lib.symgb_synchronize(uu.handle))
        barrier(world)
        t0 = time.perf_counter()
        for k in range(steps):
            step(k)
        for uu, _, _ in pipe:
            native.check(lib.symgb_synchronize(uu.handle))
        by_streams[cs] = max_over_ranks(world, (time.perf_counter() - t0) / steps)
        barrier(world)
    copy_streams = min(by_streams, key=by_streams.get)
    t_e2e = by_streams[copy_streams]
    got = pipe[1][2].numpy().reshape(S, -1)
    err = max(err, max(rel_err(got[s], w.numeric, floor) for s in (0, S - 1)))
    u2.close()
    return {"value": world * nnz * S / t_e2e, "unit": "nnz/s", "ms_per_step": t_e2e * 1e3,
            "h2d_bytes_per_step": int(sum(a.nbytes for a in inputs)), "d2h_bytes_per_step": int(nnz * S * 8),
            "steps": steps, "max_rel_err_vs_fp64_model": err,
            "mode": "two units on two streams take alternate steps (async set_arg / run / get_result: results "
                    "gathered on the device and copied to page-locked memory on the unit's copy stream); every "
                    "step copies its inputs in and its results out; no L2 clearing",
            "copy_streams": copy_streams,
            "ms_per_step_by_copy_streams": {str(k): v * 1e3 for k, v in by_streams.items()},
            "one_at_a_time": {"value": world * nnz * S / t_seq, "ms_per_step": t_seq * 1e3}}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        main_engine(args)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
