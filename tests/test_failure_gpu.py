"""Failure handling of the bounded grid barrier, made to fail from the host.

The persistent schedule (and the interpreter's fused levels) separate levels
by a grid barrier whose every wait is bounded by the device timer.  Here the
host asks each barrier to wait for one arrival more than the grid has, with a
limit of a few milliseconds: every block gives up, records the timeout and
returns, and the run reports SYMGB_ERR_TIMEOUT.  The context stays usable: the
same unit then runs normally and its results are bit-identical to the
reference's.  No fault, no unbounded wait."""
import time

import numpy as np
import pytest

from conftest import load_golden
from symboliclib_gb300 import native

pytestmark = pytest.mark.gpu

TIMEOUT = -4  # SYMGB_ERR_TIMEOUT


def inputs(w, flat):
    out, off = [], 0
    for a in w.inputs:
        out.append(flat[off:off + len(a)])
        off += len(a)
    return out


@pytest.mark.parametrize("executor,kind,depth", [
    (native.EXEC_COMPILED, native.SCHEDULE_PERSISTENT, 0),
    (native.EXEC_INTERPRETER, native.SCHEDULE_PERSISTENT, 0),
    (native.EXEC_INTERPRETER, native.SCHEDULE_LEVELS, 2),
])
def test_barrier_timeout_is_reported_and_recovered(executor, kind, depth):
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w)
    lib = native.symgb()
    u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor, fusion_depth=depth)
    for i, a in enumerate(inputs(w, inp)):
        u.set_arg(i, a)
    u.set_barrier_limits(3_000_000, extra_arrivals=1)  # 3 ms, one arrival that never comes
    t0 = time.perf_counter()
    rc = lib.symgb_run(u.handle)
    elapsed = time.perf_counter() - t0
    assert rc == TIMEOUT, lib.symgb_last_error().decode()
    assert b"timed out" in lib.symgb_last_error()
    assert elapsed < 5.0
    # The same unit with the normal limits runs and is exact.
    u.set_barrier_limits(2_000_000_000, extra_arrivals=0)
    for _ in range(2):
        u.run()
        assert np.array_equal(u.get_result(0).view(np.uint64), gold.view(np.uint64))
