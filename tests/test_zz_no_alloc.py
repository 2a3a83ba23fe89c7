"""GPU test of the allocation-free entry point, symgb_run_static.

It serves callers that cannot allocate device memory themselves (a framework
that owns all device memory through its own pool, or code that must not
allocate once running): they pass device buffers for inputs and outputs, and
the engine keeps all working memory in one static device array.  Its results
must equal those of the normal entry points (symgb_init / symgb_set_arg /
symgb_run / symgb_get_result) on the same plan, bit for bit in exact mode (the
tolerance of the parity tests), on two calls in a row.  This file is collected
last so that a run stopping at its first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from symboliclib_gb300 import native

pytestmark = pytest.mark.gpu


def reference_result(w):
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=native.SCHEDULE_PERSISTENT, math=native.MATH_EXACT)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, a)
    u.run()
    return u.get_result(0)


def static_unit(w):
    lib = native.symgb()
    h = C.c_void_p()
    native.check(lib.symgb_unit_create(w.plan, C.byref(h)))
    s = native.Schedule(native.SCHEDULE_PERSISTENT, native.MATH_EXACT, 0, 0, 0, 0, 1, 0)
    native.check(lib.symgb_set_schedule(h, C.byref(s)))
    return lib, h


def run_static(lib, h, w, inputs_dev, outputs_dev):
    import torch
    ins = (C.c_void_p * len(inputs_dev))(*[t.data_ptr() for t in inputs_dev])
    outs = (C.c_void_p * len(outputs_dev))(*[t.data_ptr() for t in outputs_dev])
    idx = np.ascontiguousarray(w.index_data, np.uint32)
    ids = np.ascontiguousarray(w.out_index_data, np.uint32)
    cst = np.ascontiguousarray(w.const_data if len(w.const_data) else np.zeros(1), np.float64)
    stream = torch.cuda.current_stream().cuda_stream
    return lib.symgb_run_static(h, idx.ctypes.data, ids.ctypes.data, cst.ctypes.data, ins, outs, C.c_void_p(stream))


@pytest.mark.parametrize("name,size,seed", [("cotan", 24, 3), ("cloth", 8, 4), ("ata", 12, 5)])
def test_static_entry_matches_normal_entry(name, size, seed):
    import torch
    w = native.Workload(name, size, seed)
    ref = reference_result(w)
    lib, h = static_unit(w)
    try:
        inputs_dev = [torch.from_numpy(a).cuda() for a in w.inputs]
        outputs_dev = [torch.full((len(ref),), np.nan, dtype=torch.float64, device="cuda")]
        for call in range(2):
            native.check(run_static(lib, h, w, inputs_dev, outputs_dev))
            out = outputs_dev[0].cpu().numpy()
            assert np.array_equal(out.view(np.uint64), ref.view(np.uint64)), f"call {call}"
            outputs_dev[0].fill_(np.nan)
        # a different input after the first two calls: still the normal path's result
        scaled = [a * 1.25 for a in w.inputs]
        inputs2 = [torch.from_numpy(a).cuda() for a in scaled]
        native.check(run_static(lib, h, w, inputs2, outputs_dev))
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
        for i, a in enumerate(scaled):
            u.set_arg(i, a)
        u.run()
        assert np.array_equal(outputs_dev[0].cpu().numpy().view(np.uint64), u.get_result(0).view(np.uint64))
    finally:
        lib.symgb_unit_destroy(h)


def test_static_entry_allocates_no_device_memory():
    """Once the first call has loaded the module (and with it the static
    array), further calls leave the device's free memory unchanged."""
    import torch
    w = native.Workload("cloth", 8, 4)
    lib, h = static_unit(w)
    try:
        inputs_dev = [torch.from_numpy(a).cuda() for a in w.inputs]
        outputs_dev = [torch.empty(len(w.numeric), dtype=torch.float64, device="cuda")]
        native.check(run_static(lib, h, w, inputs_dev, outputs_dev))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for _ in range(3):
            native.check(run_static(lib, h, w, inputs_dev, outputs_dev))
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] >= free_before
    finally:
        lib.symgb_unit_destroy(h)


def test_static_entry_rejects_plans_beyond_its_scratch():
    import torch
    w = native.Workload("cotan", 8, 1)
    # Declare an x of 5M doubles (40 MB): the plan is still valid, but its
    # working memory exceeds the entry point's 32 MiB array.
    w.plan.contents.num_total_memory = 5_000_000
    lib, h = static_unit(w)
    try:
        inputs_dev = [torch.from_numpy(a).cuda() for a in w.inputs]
        outputs_dev = [torch.empty(len(w.numeric), dtype=torch.float64, device="cuda")]
        rc = run_static(lib, h, w, inputs_dev, outputs_dev)
        assert rc == -1
        assert b"bytes of scratch" in lib.symgb_last_error()
    finally:
        lib.symgb_unit_destroy(h)
