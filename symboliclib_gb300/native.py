"""ctypes bindings of the engine's C ABI (include/symgb.h) and of the workload
library.  The device path is native code only: if the libraries are missing
this module raises instead of falling back to anything else."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "lib"

SCHEDULE_PLAIN, SCHEDULE_LEVELS, SCHEDULE_PERSISTENT = 0, 1, 2
MATH_EXACT, MATH_FAST = 0, 1
EXEC_COMPILED, EXEC_INTERPRETER = 0, 1
LOAD_READONLY, LOAD_L1, LOAD_L2 = 0, 1, 2
ITEMS_STRIDED, ITEMS_GROUPED = 0, 1


class Node(C.Structure):
    _fields_ = [("op", C.c_int32), ("nchild", C.c_int32), ("a", C.c_int32), ("b", C.c_int32), ("value", C.c_double)]


class KernelDesc(C.Structure):
    _fields_ = [("num_instances", C.c_uint64), ("output_offset", C.c_uint64), ("index_offset", C.c_uint64),
                ("constants_offset", C.c_uint64), ("num_output_rows", C.c_uint32), ("num_index_rows", C.c_uint32),
                ("num_constant_rows", C.c_uint32), ("level", C.c_int32), ("num_nodes", C.c_uint32),
                ("nodes", C.POINTER(Node)), ("num_access", C.c_uint32), ("access", C.POINTER(C.c_int32))]


class PlanDesc(C.Structure):
    _fields_ = [("num_kernels", C.c_uint32), ("kernels", C.POINTER(KernelDesc)), ("num_args", C.c_uint32),
                ("arg_start", C.POINTER(C.c_uint64)), ("arg_length", C.POINTER(C.c_uint64)),
                ("num_outputs", C.c_uint32), ("output_start", C.POINTER(C.c_uint64)),
                ("output_length", C.POINTER(C.c_uint64)), ("num_total_memory", C.c_uint64),
                ("num_indices", C.c_uint64), ("num_output_values", C.c_uint64), ("num_constants", C.c_uint64),
                ("threads_per_block", C.c_uint32)]


class Schedule(C.Structure):
    _fields_ = [("kind", C.c_int32), ("math", C.c_int32), ("threads_per_block", C.c_int32),
                ("items_per_tile", C.c_int32), ("blocks_per_sm", C.c_int32), ("use_graph", C.c_int32),
                ("items_per_thread", C.c_int32), ("fusion_depth", C.c_int32), ("lanes_per_item", C.c_int32),
                ("executor", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("num_kernels", "num_levels", "num_inputs", "num_outputs",
                                           "num_intermediates", "index_entries", "constant_entries", "flops",
                                           "divs", "sqrts", "transcendentals", "gathers", "max_registers",
                                           "program_words", "bundles", "bundle_entries")]


# Every function declared in include/symgb.h, with its ctypes signature.
SYMGB_FUNCTIONS = {
    "symgb_unit_create": (C.c_int, [C.POINTER(PlanDesc), C.POINTER(C.c_void_p)]),
    "symgb_init": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "symgb_set_arg": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_run": (C.c_int, [C.c_void_p]),
    "symgb_get_result": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_finish": (C.c_int, [C.c_void_p]),
    "symgb_unit_destroy": (None, [C.c_void_p]),
    "symgb_last_error": (C.c_char_p, []),
    "symgb_set_schedule": (C.c_int, [C.c_void_p, C.POINTER(Schedule)]),
    "symgb_get_schedule": (C.c_int, [C.c_void_p, C.POINTER(Schedule)]),
    "symgb_set_num_sets": (C.c_int, [C.c_void_p, C.c_int]),
    "symgb_num_sets": (C.c_int, [C.c_void_p]),
    "symgb_set_arg_sets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_get_result_sets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "symgb_run_async": (C.c_int, [C.c_void_p]),
    "symgb_set_arg_sets_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_get_result_sets_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_synchronize": (C.c_int, [C.c_void_p]),
    "symgb_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "symgb_algorithmic_bytes": (C.c_uint64, [C.c_void_p, C.c_int]),
    "symgb_last_launch_count": (C.c_int, [C.c_void_p]),
    "symgb_run_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "symgb_measure_fp64_rate": (C.c_int, [C.POINTER(C.c_double)]),
    "symgb_set_kernel_shape": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "symgb_set_arg_sets_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_get_result_sets_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "symgb_solver_create": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "symgb_solver_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                     C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "symgb_solver_multiply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "symgb_solver_destroy": (None, [C.c_void_p]),
    "symgb_solver_set_block_preconditioner": (C.c_int, [C.c_void_p, C.c_int, C.c_int64]),
    "symgb_time_kernels": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_uint64, C.POINTER(C.c_double)]),
    "symgb_plan_save": (C.c_int, [C.c_char_p, C.POINTER(PlanDesc), C.c_void_p, C.c_void_p, C.c_void_p]),
    "symgb_plan_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "symgb_plan_file_desc": (C.POINTER(PlanDesc), [C.c_void_p]),
    "symgb_plan_file_index_data": (C.POINTER(C.c_uint32), [C.c_void_p]),
    "symgb_plan_file_out_index_data": (C.POINTER(C.c_uint32), [C.c_void_p]),
    "symgb_plan_file_const_data": (C.POINTER(C.c_double), [C.c_void_p]),
    "symgb_plan_file_free": (None, [C.c_void_p]),
    "symgb_plan_last_error": (C.c_char_p, []),
    "symgb_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "symgb_batch_run": (C.c_int, [C.c_void_p]),
    "symgb_batch_run_async": (C.c_int, [C.c_void_p, C.c_void_p]),
    "symgb_batch_launch_count": (C.c_int, [C.c_void_p]),
    "symgb_batch_destroy": (None, [C.c_void_p]),
    "symgb_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "symgb_mlp_num_params": (C.c_int, [C.c_void_p]),
    "symgb_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "symgb_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "symgb_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "symgb_mlp_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_float)]),
    "symgb_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float,
                                  C.POINTER(C.c_float)]),
    "symgb_mlp_destroy": (None, [C.c_void_p]),
    "symgb_prepare": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "symgb_compiled_source": (C.c_int64, [C.c_void_p, C.c_int, C.c_char_p, C.c_uint64]),
    "symgb_compile_check": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "symgb_set_barrier_limits": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int]),
    "symgb_set_copy_streams": (C.c_int, [C.c_void_p, C.c_int]),
    "symgb_compiled_registers": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "symgb_set_load_path": (C.c_int, [C.c_void_p, C.c_int]),
    "symgb_set_item_layout": (C.c_int, [C.c_void_p, C.c_int]),
    "symgb_set_direct_outputs": (C.c_int, [C.c_void_p, C.c_int]),
    "symgb_kernel_program": (C.c_int64, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_uint64, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
}

_libs: dict[str, C.CDLL] = {}


def _load(name: str) -> C.CDLL:
    if name not in _libs:
        path = LIB_DIR / f"lib{name}.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it with `python -m symboliclib_gb300.build`")
        _libs[name] = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
    return _libs[name]


def symgb() -> C.CDLL:
    lib = _load("symgb")
    if not getattr(lib, "_typed", False):
        for fn, (res, args) in SYMGB_FUNCTIONS.items():
            f = getattr(lib, fn)
            f.restype = res
            f.argtypes = args
        lib._typed = True
    return lib


def workloads() -> C.CDLL:
    symgb()
    lib = _load("symgb_workloads")
    if not getattr(lib, "_typed", False):
        lib.symgbw_build.restype = C.c_int
        lib.symgbw_build.argtypes = [C.c_char_p, C.c_int, C.c_ulonglong, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        lib.symgbw_last_error.restype = C.c_char_p
        lib.symgbw_free.argtypes = [C.c_void_p]
        lib.symgbw_plan.restype = C.POINTER(PlanDesc)
        lib.symgbw_plan.argtypes = [C.c_void_p]
        for fn in ("symgbw_index_data", "symgbw_out_index_data"):
            getattr(lib, fn).restype = C.POINTER(C.c_uint32)
            getattr(lib, fn).argtypes = [C.c_void_p]
        lib.symgbw_const_data.restype = C.POINTER(C.c_double)
        lib.symgbw_const_data.argtypes = [C.c_void_p]
        lib.symgbw_num_inputs.argtypes = [C.c_void_p]
        lib.symgbw_input.restype = C.POINTER(C.c_double)
        lib.symgbw_input.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]
        lib.symgbw_numeric.restype = C.POINTER(C.c_double)
        lib.symgbw_numeric.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        lib.symgbw_plan_text.restype = C.c_uint64
        lib.symgbw_plan_text.argtypes = [C.c_void_p, C.c_char_p, C.c_uint64]
        lib.symgbw_front_seconds.restype = C.c_double
        lib.symgbw_front_seconds.argtypes = [C.c_void_p]
        lib.symgbw_model_seconds.restype = C.c_double
        lib.symgbw_model_seconds.argtypes = [C.c_void_p]
        lib.symgbw_pattern.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.POINTER(C.c_int))]
        lib._typed = True
    return lib


def check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(f"symgb error {rc}: {symgb().symgb_last_error().decode()}")


def _array(ptr, n: int, dtype) -> np.ndarray:
    """Copy of n elements behind a ctypes pointer (empty when n is 0)."""
    if n == 0:
        return np.empty(0, dtype)
    return np.ctypeslib.as_array(ptr, (int(n),)).copy()


class Workload:
    """A synthetic workload planned by the engine's front end."""

    def __init__(self, name: str, size: int, seed: int, vector_width: int = 0, text: bool = False):
        lib = workloads()
        h = C.c_void_p()
        if lib.symgbw_build(name.encode(), size, seed, vector_width, int(text), C.byref(h)) != 0:
            raise RuntimeError(f"workload {name}: {lib.symgbw_last_error().decode()}")
        self._lib, self.handle = lib, h
        self.name, self.size, self.seed = name, size, seed
        self.plan = lib.symgbw_plan(h)
        d = self.plan.contents
        self.num_total_memory = int(d.num_total_memory)
        self.index_data = _array(lib.symgbw_index_data(h), d.num_indices, np.uint32)
        self.out_index_data = _array(lib.symgbw_out_index_data(h), d.num_output_values, np.uint32)
        self.const_data = _array(lib.symgbw_const_data(h), d.num_constants, np.float64)
        self.inputs = []
        for i in range(lib.symgbw_num_inputs(h)):
            n = C.c_uint64()
            p = lib.symgbw_input(h, i, C.byref(n))
            self.inputs.append(_array(p, n.value, np.float64))
        n = C.c_uint64()
        p = lib.symgbw_numeric(h, C.byref(n))
        self.numeric = _array(p, n.value, np.float64)
        self.front_seconds = lib.symgbw_front_seconds(h)  # model construction + planning
        self.model_seconds = lib.symgbw_model_seconds(h)  # model construction alone

    def pattern(self):
        """(rows, cols, col_ptr, row_idx) of the output matrix in CSC form."""
        rows, cols = C.c_int(), C.c_int()
        cp, ri = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
        self._lib.symgbw_pattern(self.handle, C.byref(rows), C.byref(cols), C.byref(cp), C.byref(ri))
        col_ptr = _array(cp, cols.value + 1, np.int32).astype(np.int64) if cols.value else np.zeros(1, np.int64)
        row_idx = _array(ri, int(col_ptr[-1]), np.int32)
        return rows.value, cols.value, col_ptr, row_idx

    @property
    def plan_text(self) -> str:
        n = self._lib.symgbw_plan_text(self.handle, None, 0)
        buf = C.create_string_buffer(int(n) + 1)
        self._lib.symgbw_plan_text(self.handle, buf, n + 1)
        return buf.value.decode()

    @property
    def arg_start(self) -> list[int]:
        d = self.plan.contents
        return [int(d.arg_start[i]) for i in range(d.num_args)]

    @property
    def output_length(self) -> list[int]:
        d = self.plan.contents
        return [int(d.output_length[i]) for i in range(d.num_outputs)]

    def __del__(self):
        try:
            self._lib.symgbw_free(self.handle)
        except Exception:
            pass


def save_plan(path, plan: C.POINTER(PlanDesc), index_data, out_index_data, const_data) -> None:
    """Writes a plan and its tables to a versioned plan file (symgb_plan_save)."""
    lib = symgb()
    tables = [np.ascontiguousarray(index_data, np.uint32), np.ascontiguousarray(out_index_data, np.uint32),
              np.ascontiguousarray(const_data, np.float64)]
    if lib.symgb_plan_save(str(path).encode(), plan, *(t.ctypes.data for t in tables)) != 0:
        raise RuntimeError(lib.symgb_plan_last_error().decode())


class PlanFile:
    """A plan read back from a plan file (symgb_plan_load); the same fields as
    a Workload's plan and tables, valid while this object lives."""

    def __init__(self, path):
        lib = symgb()
        h = C.c_void_p()
        if lib.symgb_plan_load(str(path).encode(), C.byref(h)) != 0:
            raise RuntimeError(lib.symgb_plan_last_error().decode())
        self._lib, self.handle = lib, h
        self.plan = lib.symgb_plan_file_desc(h)
        d = self.plan.contents
        self.index_data = _array(lib.symgb_plan_file_index_data(h), d.num_indices, np.uint32)
        self.out_index_data = _array(lib.symgb_plan_file_out_index_data(h), d.num_output_values, np.uint32)
        self.const_data = _array(lib.symgb_plan_file_const_data(h), d.num_constants, np.float64)

    def __del__(self):
        if getattr(self, "handle", None):
            self._lib.symgb_plan_file_free(self.handle)
            self.handle = None


SOLVER_CG, SOLVER_BICGSTAB = 0, 1


class SparseSolver:
    """Batched Jacobi-preconditioned Krylov solves (symgb_solver_*) for S
    symmetric systems sharing one CSC pattern: conjugate gradient (positive
    definite) or BiCGSTAB (indefinite); solve and multiply take torch CUDA
    tensors (values [S, nnz], vectors [S, n])."""

    def __init__(self, n: int, col_ptr, row_idx, lower_only: bool = True, num_sets: int = 1):
        lib = symgb()
        self._cp = np.ascontiguousarray(col_ptr, np.int64)
        self._ri = np.ascontiguousarray(row_idx, np.int32)
        h = C.c_void_p()
        check(lib.symgb_solver_create(n, self._cp.ctypes.data, self._ri.ctypes.data, int(lower_only), num_sets,
                                      C.byref(h)))
        self._lib, self.handle, self.n, self.num_sets = lib, h, n, num_sets

    def solve(self, values, b, x, tol: float = 1e-10, max_iter: int = 1000, method: int = SOLVER_CG, stream=None):
        """Returns (iterations, largest relative residual over the systems)."""
        it, res = C.c_int(), C.c_double()
        st = C.c_void_p(stream.cuda_stream) if stream is not None else None
        check(self._lib.symgb_solver_solve(self.handle, method, C.c_void_p(values.data_ptr()), C.c_void_p(b.data_ptr()),
                                           C.c_void_p(x.data_ptr()), tol, max_iter, st, C.byref(it), C.byref(res)))
        return it.value, res.value

    def set_block_preconditioner(self, block_size: int, stride: int) -> None:
        """BiCGSTAB with block Jacobi (symgb_solver_set_block_preconditioner)."""
        check(self._lib.symgb_solver_set_block_preconditioner(self.handle, block_size, stride))

    def multiply(self, values, p, q, stream=None) -> None:
        st = C.c_void_p(stream.cuda_stream) if stream is not None else None
        check(self._lib.symgb_solver_multiply(self.handle, C.c_void_p(values.data_ptr()), C.c_void_p(p.data_ptr()),
                                              C.c_void_p(q.data_ptr()), st))

    def __del__(self):
        if getattr(self, "handle", None):
            self._lib.symgb_solver_destroy(self.handle)
            self.handle = None


class Unit:
    """One engine unit (device state for a plan), driven through the C ABI."""

    def __init__(self, plan: C.POINTER(PlanDesc), index_data, out_index_data, const_data, init: bool = True):
        lib = symgb()
        h = C.c_void_p()
        check(lib.symgb_unit_create(plan, C.byref(h)))
        self._lib, self.handle = lib, h
        self._tables = (np.ascontiguousarray(index_data, np.uint32), np.ascontiguousarray(out_index_data, np.uint32),
                        np.ascontiguousarray(const_data, np.float64))
        if init:  # device memory and table upload; host-only uses (sources, statistics) skip it
            check(lib.symgb_init(h, *(t.ctypes.data for t in self._tables)))
        d = plan.contents
        self.kernel_instances = [int(d.kernels[k].num_instances) for k in range(d.num_kernels)]
        self.kernel_levels = [int(d.kernels[k].level) for k in range(d.num_kernels)]
        self.arg_length = [int(d.arg_length[i]) for i in range(d.num_args)]
        self.output_length = [int(d.output_length[i]) for i in range(d.num_outputs)]

    @classmethod
    def from_workload(cls, w: Workload, init: bool = True) -> "Unit":
        return cls(w.plan, w.index_data, w.out_index_data, w.const_data, init=init)

    def set_schedule(self, kind=SCHEDULE_PLAIN, math=MATH_FAST, threads_per_block=0, items_per_tile=0,
                     blocks_per_sm=0, use_graph=0, items_per_thread=1, fusion_depth=0, lanes_per_item=1,
                     executor=EXEC_COMPILED) -> None:
        s = Schedule(kind, math, threads_per_block, items_per_tile, blocks_per_sm, use_graph, items_per_thread,
                     fusion_depth, lanes_per_item, executor)
        check(self._lib.symgb_set_schedule(self.handle, C.byref(s)))

    def prepare(self) -> float:
        """Compiles the compiled executor's module for the current schedule
        (symgb_prepare); returns the seconds spent (0 when cached)."""
        t = C.c_double()
        check(self._lib.symgb_prepare(self.handle, C.byref(t)))
        return t.value

    def compiled_source(self, kind: int) -> str:
        n = self._lib.symgb_compiled_source(self.handle, kind, None, 0)
        if n < 0:
            check(int(n))
        buf = C.create_string_buffer(int(n) + 1)
        self._lib.symgb_compiled_source(self.handle, kind, buf, n + 1)
        return buf.value.decode()

    def compile_check(self, kind: int) -> float:
        """Compiles the generated module with NVRTC (no device); returns seconds."""
        t = C.c_double()
        check(self._lib.symgb_compile_check(self.handle, kind, C.byref(t)))
        return t.value

    def set_barrier_limits(self, timeout_ns: int, extra_arrivals: int = 0) -> None:
        check(self._lib.symgb_set_barrier_limits(self.handle, timeout_ns, extra_arrivals))

    def set_num_sets(self, n: int) -> None:
        check(self._lib.symgb_set_num_sets(self.handle, n))

    def compiled_registers(self, kind: int) -> list[int]:
        """Registers per thread of every launch of the compiled module of `kind`."""
        n = self._lib.symgb_compiled_registers(self.handle, kind, None, 0)
        if n < 0:
            check(n)
        regs = (C.c_int * max(1, n))()
        got = self._lib.symgb_compiled_registers(self.handle, kind, regs, n)
        if got < 0:
            check(got)
        return list(regs)[:n]

    def set_direct_outputs(self, on: bool) -> None:
        """Results written straight at their positions (symgb_set_direct_outputs)."""
        check(self._lib.symgb_set_direct_outputs(self.handle, int(on)))

    def set_item_layout(self, layout: int) -> None:
        """Which work items a compiled-executor thread takes (ITEMS_STRIDED, ITEMS_GROUPED)."""
        check(self._lib.symgb_set_item_layout(self.handle, layout))

    def set_load_path(self, path: int) -> None:
        """Data path of the compiled executor's loads (LOAD_READONLY, LOAD_L1, LOAD_L2)."""
        check(self._lib.symgb_set_load_path(self.handle, path))

    def set_copy_streams(self, n: int) -> None:
        """Streams the async result copy is split over (symgb_set_copy_streams)."""
        check(self._lib.symgb_set_copy_streams(self.handle, n))

    @property
    def num_kernels(self) -> int:
        return len(self.kernel_instances)

    def set_kernel_shape(self, k: int, items: int = 0, lanes: int = 0, tpb: int = 0) -> None:
        check(self._lib.symgb_set_kernel_shape(self.handle, k, items, lanes, tpb))

    def time_kernels(self, reps: int = 5, flush=None) -> np.ndarray:
        """Mean microseconds per kernel launch under the plain schedule
        (flush: a torch CUDA tensor overwritten before every repetition)."""
        out = (C.c_double * self.num_kernels)()
        ptr = C.c_void_p(flush.data_ptr()) if flush is not None else None
        nbytes = flush.numel() * flush.element_size() if flush is not None else 0
        check(self._lib.symgb_time_kernels(self.handle, reps, ptr, nbytes, out))
        return np.array(out[:])

    @property
    def num_sets(self) -> int:
        return self._lib.symgb_num_sets(self.handle)

    def set_arg(self, i: int, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, np.float64)
        if v.size != self.arg_length[i] * self.num_sets:
            raise ValueError("input size mismatch")
        check(self._lib.symgb_set_arg_sets(self.handle, v.ctypes.data, i))

    def run(self) -> None:
        check(self._lib.symgb_run(self.handle))

    def get_result(self, k: int = 0) -> np.ndarray:
        out = np.empty(self.output_length[k] * self.num_sets, np.float64)
        check(self._lib.symgb_get_result_sets(self.handle, out.ctypes.data, k))
        return out

    def stats(self) -> Stats:
        s = Stats()
        check(self._lib.symgb_get_stats(self.handle, C.byref(s)))
        return s

    def algorithmic_bytes(self, num_sets: int) -> int:
        return int(self._lib.symgb_algorithmic_bytes(self.handle, num_sets))

    def last_launch_count(self) -> int:
        return self._lib.symgb_last_launch_count(self.handle)

    def close(self) -> None:
        if self.handle:
            self._lib.symgb_unit_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """The engine's FP32 cost-model network (include/symgb.h, symgb_mlp_*)."""

    def __init__(self, inputs: int, hidden: int = 64, seed: int = 0):
        self._lib = symgb()
        h = C.c_void_p()
        check(self._lib.symgb_mlp_create(inputs, hidden, seed, C.byref(h)))
        self.handle, self.inputs, self.hidden = h, inputs, hidden

    @property
    def num_params(self) -> int:
        return self._lib.symgb_mlp_num_params(self.handle)

    def params(self) -> np.ndarray:
        p = np.empty(self.num_params, np.float32)
        check(self._lib.symgb_mlp_get_params(self.handle, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(self._lib.symgb_mlp_set_params(self.handle, p.ctypes.data))

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        y = np.empty(len(X), np.float32)
        check(self._lib.symgb_mlp_forward(self.handle, X.ctypes.data, len(X), y.ctypes.data))
        return y

    def gradient(self, X: np.ndarray, y: np.ndarray) -> tuple[np.ndarray, float]:
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.empty(self.num_params, np.float32)
        loss = C.c_float()
        check(self._lib.symgb_mlp_gradient(self.handle, X.ctypes.data, y.ctypes.data, len(X), g.ctypes.data,
                                           C.byref(loss)))
        return g, loss.value

    def train(self, X: np.ndarray, y: np.ndarray, epochs: int, lr: float = 1e-3) -> float:
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = C.c_float()
        check(self._lib.symgb_mlp_train(self.handle, X.ctypes.data, y.ctypes.data, len(X), epochs, lr,
                                        C.byref(loss)))
        return loss.value

    def close(self) -> None:
        if self.handle:
            self._lib.symgb_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
