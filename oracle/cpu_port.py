"""CPU port of the reference's CPU ComputeUnit (TEST / BASELINE INFRASTRUCTURE).

The reference's CPU device generates one C++ function per kernel - an OpenMP
`parallel for` over instances whose body is the template's statements
(src/ComputeUnit.cpp:368-450 with src/StringResources.h:312-480) - compiles it
with `-O3 -ffast-math` and calls the kernels in order from run().  This module
generates the same structure from an engine plan (SoA table layout, pack
length 0) and compiles it with gcc -O3 -ffast-math -fopenmp.  It is what
bench.py times as the CPU baseline ("kind": "port") on machines where the
reference library itself cannot be built.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import struct
import subprocess
import time
from pathlib import Path

import numpy as np

BUILD = Path(__file__).resolve().parent / "_build"

N_CONST, N_VAR, N_ADD, N_MUL, N_MULC, N_DIV, N_SQRT = 1, 2, 3, 4, 5, 6, 7
N_NEG, N_DEFINE, N_BLOCK, N_ASSIGN, N_REC = 23, 24, 25, 18, 26
FUNCS = {8: "sin", 9: "cos", 10: "tan", 12: "asin", 13: "acos", 14: "atan", 15: "exp", 16: "log"}


def _tree(nodes):
    kids, stack = [], []
    for j, nd in enumerate(nodes):
        nc = nd.nchild
        kids.append(stack[len(stack) - nc:] if nc else [])
        if nc:
            del stack[len(stack) - nc:]
        stack.append(j)
    return kids, stack[-1]


def _literal(v: float) -> str:
    return float(v).hex()


def kernel_source(kd, k: int) -> str:
    n = int(kd.num_instances)
    nodes = [kd.nodes[j] for j in range(kd.num_nodes)]
    access = [(kd.access[2 * a], kd.access[2 * a + 1]) for a in range(kd.num_access)]
    kids, root = _tree(nodes)

    def expr(j):
        nd = nodes[j]
        if nd.op == N_CONST:
            return _literal(nd.value)
        if nd.op == N_VAR:
            if nd.b == -3:
                base, off = access[nd.a]
                return f"x[(long)p[{n * base}L + i] + ({off})]"
            if nd.b == -4:
                return f"c[{n * nd.a}L + i]"
            if nd.b == 253:
                return f"r{nd.a}"
            raise ValueError("unsupported variable group")
        cs = [expr(c) for c in kids[j]]
        if nd.op == N_ADD:
            return "(" + " + ".join(cs) + ")"
        if nd.op in (N_MUL, N_MULC):
            return "(" + " * ".join(cs) + ")"
        if nd.op == N_DIV:
            return f"({cs[0]} / {cs[1]})"
        if nd.op == N_NEG:
            return f"(-{cs[0]})"
        if nd.op == N_SQRT:
            return f"sqrt({cs[0]})"
        if nd.op == N_REC:
            return f"(1.0 / {cs[0]})"
        if nd.op == 17:
            return f"pow({cs[0]}, {cs[1]})"
        if nd.op in FUNCS:
            return f"{FUNCS[nd.op]}({cs[0]})"
        raise ValueError(f"unsupported operation {nd.op}")

    lines = []

    def stmt(j):
        nd = nodes[j]
        if nd.op == N_BLOCK:
            for c in kids[j]:
                stmt(c)
            return
        lhs, rhs = kids[j]
        name = nodes[lhs]
        if nd.op == N_DEFINE:
            lines.append(f"const double r{name.a} = {expr(rhs)};")
        elif nd.op == N_ASSIGN:
            lines.append(f"y[{n * name.a}L + i] = {expr(rhs)};")
        else:
            raise ValueError("statement is neither DEFINE nor ASSIGN")

    if nodes[root].op == N_BLOCK:
        for c in kids[root]:
            stmt(c)
    else:
        stmt(root)
    body = "\n        ".join(lines)
    return (f"static void k{k}(const double* restrict x, const double* restrict c, double* y, "
            f"const unsigned* restrict p) {{\n"
            f"    #pragma omp parallel for schedule(static)\n"
            f"    for (long i = 0; i < {n}L; ++i) {{\n        {body}\n    }}\n}}\n")


def plan_source(plan) -> str:
    d = plan.contents
    parts = ["#include <math.h>\n"]
    calls = []
    for k in range(d.num_kernels):
        kd = d.kernels[k]
        parts.append(kernel_source(kd, k))
        calls.append(f"    k{k}(x, c + {int(kd.constants_offset)}L, x + {int(kd.output_offset)}L, "
                     f"p + {int(kd.index_offset)}L);")
    parts.append("void port_run(double* x, const unsigned* p, const double* c) {\n" + "\n".join(calls) + "\n}\n")
    return "\n".join(parts)


class CpuPort:
    """A compiled CPU port of one plan."""

    def __init__(self, plan, index_data, out_index_data, const_data, threads: int | None = None):
        src = plan_source(plan)
        key = hashlib.sha1(src.encode()).hexdigest()[:16]
        BUILD.mkdir(parents=True, exist_ok=True)
        so = BUILD / f"port_{key}.so"
        if not so.exists():
            c = BUILD / f"port_{key}.c"
            c.write_text(src)
            subprocess.run(["gcc", "-O3", "-ffast-math", "-fopenmp", "-fPIC", "-shared", "-std=c99",
                            str(c), "-o", str(so), "-lm"], check=True)
        self.threads = threads or os.cpu_count() or 1
        os.environ["OMP_NUM_THREADS"] = str(self.threads)
        self.lib = C.CDLL(str(so))
        self.lib.port_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        d = plan.contents
        self.arg_start = [int(d.arg_start[i]) for i in range(d.num_args)]
        self.arg_length = [int(d.arg_length[i]) for i in range(d.num_args)]
        self.out_start = [int(d.output_start[i]) for i in range(d.num_outputs)]
        self.out_length = [int(d.output_length[i]) for i in range(d.num_outputs)]
        self.x = np.zeros(max(1, d.num_total_memory), np.float64)
        self.p = np.ascontiguousarray(index_data, np.uint32)
        self.c = np.ascontiguousarray(const_data if len(const_data) else np.zeros(1), np.float64)
        self.ids = np.ascontiguousarray(out_index_data, np.int64)

    def execute(self, inputs) -> None:
        """setArg for every input container, then run() (the reference's execute())."""
        for s, n, v in zip(self.arg_start, self.arg_length, inputs):
            self.x[s:s + n] = v
        self.lib.port_run(self.x.ctypes.data, self.p.ctypes.data, self.c.ctypes.data)

    def result(self, k: int = 0) -> np.ndarray:
        s, n = self.out_start[k], self.out_length[k]
        return self.x[self.ids[s:s + n]]

    def time_execute(self, inputs, budget_s: float = 15.0, max_runs: int = 50) -> tuple[float, int]:
        """Median seconds per execute() over a bounded sample; returns (median, runs)."""
        self.execute(inputs)  # warm-up (page-in, thread start)
        times = []
        t_end = time.perf_counter() + budget_s
        while len(times) < max_runs and (len(times) < 3 or time.perf_counter() < t_end):
            t0 = time.perf_counter()
            self.execute(inputs)
            times.append(time.perf_counter() - t0)
        return float(np.median(times)), len(times)
