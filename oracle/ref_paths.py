"""The reference's own execution paths, built from the source its ComputeUnit
generated (TEST / BASELINE INFRASTRUCTURE).

oracle/ref_generate.sh runs the reference library (oracle/_ref/libsymref.so,
built from the reference's sources where they are mounted) on the project's
workloads and keeps, per workload, size and device, what the reference
writes: its generated source (cudaCode.cu for Device(UseCuda(),
ThreadsPerBlock(128)), cpuCode.cpp for Device(VecWidth(4))), its table files
(indexData, constData, outIndexData) and the inputs, in
oracle/_ref/gen/<workload>_<size>_<cuda|cpu>/.  Those directories travel to
the machine with the GPU, where oracle/ref_paths.sh compiles the sources (the reference's
own nvcc / clang++ command lines; g++ stands in for clang++) and
oracle/ref_run.cpp loads the library through the reference's five calls and
times it.  bench.py uses this for its reference arm (the CPU ComputeUnit) and
for the reference's plain GPU path; tests/ use it for parity.
"""
from __future__ import annotations

import json
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
GEN = HERE / "_ref" / "gen"
TABLES = ("indexData", "constData", "outIndexData", "inputs.bin")


def gen_dir(workload: str, size: int, device: str) -> Path:
    return GEN / f"{workload}_{size}_{device}"


def available(workload: str, size: int, device: str) -> bool:
    d = gen_dir(workload, size, device)
    src = d / ("cudaCode.cu" if device == "cuda" else "cpuCode.cpp")
    return src.is_file() and all((d / t).is_file() for t in TABLES)


def build(workload: str, size: int, device: str, threads: int | None = None) -> Path:
    """Compiles the generated source (and the timing driver) on this machine."""
    d = gen_dir(workload, size, device)
    env = dict(os.environ)
    if threads:
        env["NUMTHREADS"] = str(threads)
    r = subprocess.run(["sh", str(HERE / "ref_paths.sh"), str(d), device], capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"building the reference's {device} path failed:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    return d


def run(workload: str, size: int, device: str, library: str, warmup: int, steps: int,
        results: Path | None = None) -> dict:
    """Runs one built library of the reference's generated code (ref_run);
    returns its JSON line (median run_ms / execute_ms, run_event_ms on CUDA)."""
    d = gen_dir(workload, size, device)
    exe = d / ("ref_run" if device == "cuda" else "ref_run_cpu")
    cmd = [str(exe), str(d), str(d / library), str(warmup), str(steps)]
    if results is not None:
        cmd.append(str(results))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference {device} run failed: {r.stderr[-2000:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_execute(workload: str, size: int, budget_s: float, max_steps: int, threads: int | None = None) -> dict:
    """The reference CPU ComputeUnit (VecWidth(4), NUMTHREADS = threads or the
    host's cores): execute() = setArg + run timed as a median over a sample
    bounded to about `budget_s` seconds."""
    threads = threads or os.cpu_count() or 1
    build(workload, size, "cpu", threads)
    probe = run(workload, size, "cpu", "ref_cpu.so", 1, 3)
    per = max(probe["execute_ms"], 1e-3) * 1e-3
    steps = int(max(5, min(max_steps, budget_s / (2.5 * per))))
    res = run(workload, size, "cpu", "ref_cpu.so", 3, steps)
    res["threads"] = threads
    return res


def gpu_paths(workload: str, size: int, warmup: int, steps: int, results_dir: Path | None = None) -> dict:
    """The reference's plain GPU path (its generated CUDA, one launch per
    kernel, one value set per run) built three ways: the reference's own nvcc
    command (no -arch: compute_75 PTX JIT-compiled by the driver), with
    -arch=sm_103a, and -arch=sm_103a --fmad=false (operations rounded as
    written).  Returns run() medians (host clock including the reference's
    stream synchronisation, and CUDA events on its stream)."""
    build(workload, size, "cuda")
    out = {}
    for lib in ("ref_default", "ref_sm103a", "ref_exact"):
        res = None if results_dir is None else results_dir / f"{workload}_{size}_{lib}.bin"
        out[lib] = run(workload, size, "cuda", lib + ".so", warmup, steps, res)
    return out
