"""The reference-side binding of the C ABI.

tests/golden/gen_golden.cpp builds each fixture's plan description
(symgb_plan_desc) straight from the reference ComputeUnit's own kernel
objects and tables (buildRefPlan: the code a maintainer adds to the
reference's ComputeUnit::compile) and saves it as <name>.refplan with
symgb_plan_save.  These plans never pass through the engine's front end.
On the CPU: the file loads, and its tables, kernel offsets, instance counts
and dependency levels equal the engine front end's plan of the same
workload.  On the GPU: a unit made from it reproduces the reference's results
bit for bit in exact mode, with both executors and every schedule."""
import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, load_golden
from symboliclib_gb300 import native

SCHEDULES = [native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT]
EXECUTORS = [native.EXEC_COMPILED, native.EXEC_INTERPRETER]


def split(plan, flat):
    d = plan.contents
    return [flat[int(d.arg_start[i]):int(d.arg_start[i]) + int(d.arg_length[i])] for i in range(d.num_args)]


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_reference_plan_equals_front_end_plan(name, size, seed):
    ref = native.PlanFile(GOLDEN / f"{name}_{size}.refplan")
    w = native.Workload(name, size, seed)
    assert np.array_equal(ref.index_data, w.index_data)
    assert np.array_equal(ref.out_index_data, w.out_index_data)
    assert np.array_equal(ref.const_data.view(np.uint64), w.const_data.view(np.uint64))
    a, b = ref.plan.contents, w.plan.contents
    assert a.num_kernels == b.num_kernels and a.num_total_memory == b.num_total_memory
    for k in range(a.num_kernels):
        ka, kb = a.kernels[k], b.kernels[k]
        for f in ("num_instances", "output_offset", "index_offset", "constants_offset", "num_output_rows",
                  "num_index_rows", "num_constant_rows", "level", "num_nodes", "num_access"):
            assert getattr(ka, f) == getattr(kb, f), (k, f)
    u = native.Unit(ref.plan, ref.index_data, ref.out_index_data, ref.const_data, init=False)
    assert u.compile_check(native.SCHEDULE_LEVELS) >= 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_reference_plan_runs_bit_exact(name, size, seed):
    _, inp, gold = load_golden(name, size)
    ref = native.PlanFile(GOLDEN / f"{name}_{size}.refplan")
    u = native.Unit(ref.plan, ref.index_data, ref.out_index_data, ref.const_data)
    for executor in EXECUTORS:
        for kind in SCHEDULES:
            u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
            for i, a in enumerate(split(ref.plan, inp)):
                u.set_arg(i, a)
            u.run()
            out = u.get_result(0)
            assert np.array_equal(out.view(np.uint64), gold.view(np.uint64)), (executor, kind)
