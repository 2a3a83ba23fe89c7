"""CPU tests of the C ABI boundary: every symbol declared in include/symgb.h is
exported by the library, plans compile into device programs on the host,
invalid plans are rejected with an error code instead of reaching a kernel,
and calls out of order or with unsupported shapes return error codes."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT
from symboliclib_gb300 import native


def declared_functions():
    text = (ROOT / "include" / "symgb.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(symgb_\w+)\s*\(", text, re.M)))


def test_header_and_bindings_agree():
    assert declared_functions() == sorted(native.SYMGB_FUNCTIONS)


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(native.LIB_DIR / "libsymgb.so"))
    for fn in declared_functions():
        assert hasattr(lib, fn), fn


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_unit_create_compiles_programs(name, size, seed):
    """unit_create only plans and compiles on the host (no device calls)."""
    w = native.Workload(name, size, seed)
    lib = native.symgb()
    h = C.c_void_p()
    native.check(lib.symgb_unit_create(w.plan, C.byref(h)))
    s = native.Stats()
    native.check(lib.symgb_get_stats(h, C.byref(s)))
    d = w.plan.contents
    assert s.num_kernels == d.num_kernels
    assert s.num_outputs == d.num_output_values
    assert s.num_inputs == sum(len(a) for a in w.inputs)
    assert 0 < s.max_registers <= 255
    assert s.gathers > 0
    assert lib.symgb_algorithmic_bytes(h, 2) > lib.symgb_algorithmic_bytes(h, 1)
    # run before init is a state error, not a crash
    assert lib.symgb_run(h) == -3
    lib.symgb_unit_destroy(h)


def test_invalid_plans_are_rejected():
    w = native.Workload("cotan", 5, 21)
    lib = native.symgb()
    d = w.plan.contents
    h = C.c_void_p()
    # a kernel whose output rows would exceed x
    saved = d.kernels[0].output_offset
    d.kernels[0].output_offset = d.num_total_memory
    assert lib.symgb_unit_create(w.plan, C.byref(h)) == -1
    assert b"exceed" in lib.symgb_last_error()
    d.kernels[0].output_offset = saved
    # an unknown operation in a template
    saved_op = d.kernels[0].nodes[d.kernels[0].num_nodes - 2].op
    d.kernels[0].nodes[d.kernels[0].num_nodes - 2].op = 22  # CONDZERO
    assert lib.symgb_unit_create(w.plan, C.byref(h)) == -1
    d.kernels[0].nodes[d.kernels[0].num_nodes - 2].op = saved_op
    native.check(lib.symgb_unit_create(w.plan, C.byref(h)))
    lib.symgb_unit_destroy(h)


def test_schedule_validation():
    w = native.Workload("cotan", 5, 21)
    lib = native.symgb()
    h = C.c_void_p()
    native.check(lib.symgb_unit_create(w.plan, C.byref(h)))
    bad = native.Schedule(7, 0, 0, 0, 0, 0)
    assert lib.symgb_set_schedule(h, C.byref(bad)) == -1
    bad = native.Schedule(0, 0, 100, 0, 0, 0)  # not a multiple of 32
    assert lib.symgb_set_schedule(h, C.byref(bad)) == -1
    bad = native.Schedule(0, 0, 64, 0, 0, 0, 1, 0, 3)  # lanes per item not a power of two up to 8
    assert lib.symgb_set_schedule(h, C.byref(bad)) == -1
    ok = native.Schedule(2, 0, 64, 0, 0, 0)
    native.check(lib.symgb_set_schedule(h, C.byref(ok)))
    got = native.Schedule()
    native.check(lib.symgb_get_schedule(h, C.byref(got)))
    assert (got.kind, got.threads_per_block) == (2, 64)
    assert lib.symgb_set_num_sets(h, 0) == -1
    assert lib.symgb_set_num_sets(h, (1 << 20) + 1) == -1
    native.check(lib.symgb_set_num_sets(h, 5))
    assert lib.symgb_num_sets(h) == 5
    for call, good, bad_values in ((lib.symgb_set_copy_streams, (1, 4, 8), (0, 9)),
                                   (lib.symgb_set_load_path, (0, 1, 2), (-1, 3)),
                                   (lib.symgb_set_item_layout, (0, 1), (-1, 2)),
                                   (lib.symgb_set_direct_outputs, (0, 1), (-1, 2))):
        for v in good:
            native.check(call(h, v))
        for v in bad_values:
            assert call(h, v) == -1
    lib.symgb_unit_destroy(h)


def test_calls_before_init_and_bad_kernel_shapes_are_errors():
    """Host-side checks only: transfers, synchronisation and kernel timing
    before init are state errors, and kernel shapes outside the supported set
    are argument errors (no device call is reached)."""
    w = native.Workload("cloth", 3, 31)
    lib = native.symgb()
    h = C.c_void_p()
    native.check(lib.symgb_unit_create(w.plan, C.byref(h)))
    buf = np.zeros(64)
    assert lib.symgb_set_arg_sets_async(h, buf.ctypes.data, 0) == -3
    assert lib.symgb_get_result_sets_async(h, buf.ctypes.data, 0) == -3
    assert lib.symgb_set_arg_sets(h, buf.ctypes.data, 0) == -3
    assert lib.symgb_get_result_sets(h, buf.ctypes.data, 0) == -3
    assert lib.symgb_synchronize(h) == -3
    us = (C.c_double * 64)()
    assert lib.symgb_time_kernels(h, 1, None, 0, us) == -3
    assert lib.symgb_time_kernels(h, 0, None, 0, us) == -1
    nk = w.plan.contents.num_kernels
    assert lib.symgb_set_kernel_shape(h, nk, 1, 1, 64) == -1       # no such kernel
    assert lib.symgb_set_kernel_shape(h, 0, 3, 1, 64) == -1        # items per thread
    assert lib.symgb_set_kernel_shape(h, 0, 1, 3, 64) == -1        # lanes per item
    assert lib.symgb_set_kernel_shape(h, 0, 2, 2, 64) == -1        # lanes need one item
    assert lib.symgb_set_kernel_shape(h, 0, 1, 1, 100) == -1       # not whole warps
    native.check(lib.symgb_set_kernel_shape(h, 0, 1, 4, 128))
    native.check(lib.symgb_set_kernel_shape(h, nk - 1, 0, 0, 0))   # back to the schedule's shape
    lib.symgb_unit_destroy(h)


def test_barrier_limits_are_validated():
    """symgb_set_barrier_limits (failure tests) rejects a zero limit, negative
    extra arrivals and a null unit."""
    w = native.Workload("cotan", 5, 21)
    u = native.Unit.from_workload(w, init=False)
    lib = native.symgb()
    assert lib.symgb_set_barrier_limits(u.handle, 0, 0) == -1
    assert lib.symgb_set_barrier_limits(u.handle, 1000, -1) == -1
    assert lib.symgb_set_barrier_limits(None, 1000, 0) == -1
    assert lib.symgb_set_barrier_limits(u.handle, 1000, 0) == 0
