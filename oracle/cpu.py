"""Python side of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/liboracle.so (built from oracle/evaluate.c by
symboliclib_gb300/build.py) and evaluates a plan on the CPU in the
reference's operation order.  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, as the checker."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB = Path(__file__).resolve().parent / "_build" / "liboracle.so"
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB.exists():
            raise RuntimeError(f"{_LIB} is missing: build with `python -m symboliclib_gb300.build`")
        _lib = C.CDLL(str(_LIB))
        _lib.oracle_run.restype = C.c_int
        _lib.oracle_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.oracle_gather.restype = None
        _lib.oracle_gather.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p]
    return _lib


def evaluate(plan, index_data, out_index_data, const_data, inputs) -> list[np.ndarray]:
    """Runs every kernel of `plan` (a ctypes POINTER(PlanDesc)) for one value set
    and returns the output containers, like execute() followed by getResults()."""
    d = plan.contents
    x = np.zeros(max(1, d.num_total_memory), np.float64)
    for i, v in enumerate(inputs):
        s = int(d.arg_start[i])
        x[s:s + int(d.arg_length[i])] = v
    idx = np.ascontiguousarray(index_data, np.uint32)
    ids = np.ascontiguousarray(out_index_data, np.uint32)
    cst = np.ascontiguousarray(const_data, np.float64)
    rc = lib().oracle_run(C.cast(plan, C.c_void_p), idx.ctypes.data, cst.ctypes.data, x.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle: template it cannot evaluate")
    outs = []
    for k in range(d.num_outputs):
        n = int(d.output_length[k])
        out = np.empty(max(1, n), np.float64)
        lib().oracle_gather(x.ctypes.data, ids.ctypes.data, int(d.output_start[k]), n, out.ctypes.data)
        outs.append(out[:n])
    return outs
