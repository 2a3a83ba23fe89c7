"""Versioned plan file (symgb_plan_save / symgb_plan_load): a plan written
and read back is the same plan; damaged files are rejected."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from symboliclib_gb300 import native


def plan_fields(plan):
    d = plan.contents
    ks = []
    for k in range(d.num_kernels):
        K = d.kernels[k]
        nodes = [(K.nodes[j].op, K.nodes[j].nchild, K.nodes[j].a, K.nodes[j].b,
                  np.float64(K.nodes[j].value).view(np.uint64)) for j in range(K.num_nodes)]
        access = [K.access[j] for j in range(2 * K.num_access)]
        ks.append((K.num_instances, K.output_offset, K.index_offset, K.constants_offset, K.num_output_rows,
                   K.num_index_rows, K.num_constant_rows, K.level, nodes, access))
    return (d.num_total_memory, d.num_indices, d.num_output_values, d.num_constants, d.threads_per_block,
            [d.arg_start[i] for i in range(d.num_args)], [d.arg_length[i] for i in range(d.num_args)],
            [d.output_start[i] for i in range(d.num_outputs)], [d.output_length[i] for i in range(d.num_outputs)], ks)


def programs(plan):
    lib = native.symgb()
    h = C.c_void_p()
    native.check(lib.symgb_unit_create(plan, C.byref(h)))
    out = []
    for k in range(plan.contents.num_kernels):
        for math in (0, 1):
            r, nl = C.c_int(), C.c_int()
            n = lib.symgb_kernel_program(h, k, math, None, 0, C.byref(r), C.byref(nl))
            buf = (C.c_uint64 * n)()
            lib.symgb_kernel_program(h, k, math, buf, n, C.byref(r), C.byref(nl))
            out.append((list(buf), r.value, nl.value))
    lib.symgb_unit_destroy(h)
    return out


@pytest.mark.parametrize("name,size,seed", [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 2, 42), ("ata", 9, 12)])
def test_round_trip(tmp_path, name, size, seed):
    w = native.Workload(name, size, seed)
    path = tmp_path / f"{name}.symgbplan"
    native.save_plan(path, w.plan, w.index_data, w.out_index_data, w.const_data)
    f = native.PlanFile(path)
    assert plan_fields(f.plan) == plan_fields(w.plan)
    assert np.array_equal(f.index_data, w.index_data)
    assert np.array_equal(f.out_index_data, w.out_index_data)
    assert np.array_equal(f.const_data.view(np.uint64), w.const_data.view(np.uint64))
    assert programs(f.plan) == programs(w.plan)


def test_damaged_files_are_rejected(tmp_path):
    w = native.Workload("cotan", 5, 21)
    path = tmp_path / "p.symgbplan"
    native.save_plan(path, w.plan, w.index_data, w.out_index_data, w.const_data)
    good = path.read_bytes()
    cases = {
        "flipped byte": good[:100] + bytes([good[100] ^ 1]) + good[101:],
        "truncated": good[:-20],
        "not a plan": b"NOTAPLAN" + good[8:],
        "empty": b"",
    }
    for what, data in cases.items():
        bad = tmp_path / "bad.symgbplan"
        bad.write_bytes(data)
        with pytest.raises(RuntimeError):
            native.PlanFile(bad)
    with pytest.raises(RuntimeError):
        native.PlanFile(tmp_path / "missing.symgbplan")


@pytest.mark.gpu
def test_loaded_plan_runs_bit_exact(tmp_path):
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    path = tmp_path / "cloth.symgbplan"
    native.save_plan(path, w.plan, w.index_data, w.out_index_data, w.const_data)
    f = native.PlanFile(path)
    u = native.Unit(f.plan, f.index_data, f.out_index_data, f.const_data)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
    off = 0
    for i, a in enumerate(w.inputs):
        u.set_arg(i, inp[off:off + len(a)])
        off += len(a)
    u.run()
    assert np.array_equal(u.get_result(0).view(np.uint64), gold.view(np.uint64))
