"""The engine's program compiler on the CPU: the device programs of every
ComputeKernel (linear compile, bundling, register allocation, accumulator
forwarding, encoding), read back through the C ABI and run by a CPU model of
the interpreter (tests/program_model.py), reproduce the reference's golden
results bit for bit in exact mode and within the fast-mode tolerance in fast
mode; larger and random plans against the CPU oracle.  No GPU needed: units
are only created (programs are compiled at creation), never initialised."""
import ctypes as C

import numpy as np
import pytest

import program_model as pm
from conftest import GOLDEN_CASES, load_golden
from symboliclib_gb300 import native

import oracle.cpu as ocpu

FAST_FLOOR = {"cloth": 1e-4, "neohookean": 1e-4, "cotan": 1e-4}


def split_inputs(w, flat):
    out, off = [], 0
    for a in w.inputs:
        out.append(flat[off:off + len(a)])
        off += len(a)
    return out


def rel_err(a, ref, floor_frac=1e-10):
    floor = floor_frac * np.max(np.abs(ref))
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor)))


class Created:
    """A unit created (programs compiled) but not initialised."""

    def __init__(self, w):
        self.lib = native.symgb()
        self.h = C.c_void_p()
        native.check(self.lib.symgb_unit_create(w.plan, C.byref(self.h)))

    def __del__(self):
        self.lib.symgb_unit_destroy(self.h)


def model(w, inputs, math_mode):
    u = Created(w)
    return pm.evaluate(u.lib, u.h, w.plan, w.index_data, w.out_index_data, w.const_data, inputs, math_mode)[0]


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_exact_programs_reproduce_golden_results(name, size, seed):
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    out = model(w, split_inputs(w, inp), native.MATH_EXACT)
    assert np.array_equal(out.view(np.uint64), gold.view(np.uint64))


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_fast_programs_within_tolerance(name, size, seed):
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    out = model(w, split_inputs(w, inp), native.MATH_FAST)
    assert rel_err(out, gold, FAST_FLOOR.get(name, 1e-10)) <= 1e-12


@pytest.mark.parametrize("name,size", [("cotan", 40), ("cloth", 12), ("ata", 40), ("neohookean", 3),
                                       ("random", 3000), ("literals", 300)])
def test_exact_programs_match_oracle_on_larger_plans(name, size):
    w = native.Workload(name, size, 9)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    out = model(w, w.inputs, native.MATH_EXACT)
    assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("seed", [3, 22, 28, 41])
def test_random_plans_both_modes(seed):
    w = native.Workload("random", 2000, seed)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    assert np.array_equal(model(w, w.inputs, native.MATH_EXACT).view(np.uint64), ref.view(np.uint64))
    assert rel_err(model(w, w.inputs, native.MATH_FAST), ref) <= 1e-12


def test_model_catches_a_planted_program_error():
    """The check has teeth: a program with one register operand changed no
    longer reproduces the oracle."""
    w = native.Workload("cotan", 6, 3)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    u = Created(w)
    d = w.plan.contents
    x = np.zeros(d.num_total_memory)
    x[int(d.arg_start[0]):int(d.arg_start[0]) + int(d.arg_length[0])] = w.inputs[0]
    idx = np.ascontiguousarray(w.index_data, np.uint32)
    cst = np.ascontiguousarray(w.const_data, np.float64)
    planted = False
    for k in range(d.num_kernels):
        kd = d.kernels[k]
        n = int(kd.num_instances)
        words, _, nl = pm.kernel_program(u.lib, u.h, k, native.MATH_EXACT)
        if not planted:  # swap the operands of the first subtraction
            pc = nl
            while int(words[pc]) & 0xff:
                h = int(words[pc])
                cnt = (h >> 8) & 0xffff
                if h & 0xff == pm.OP_SUB:
                    e = int(words[pc + 1]) & 0xffffffff
                    a, b = (e >> 8) & 0xff, (e >> 16) & 0xff
                    e2 = (e & 0xff0000ff) | (b << 8) | (a << 16)
                    words[pc + 1] = np.uint64((int(words[pc + 1]) & ~0xffffffff) | e2)
                    planted = True
                    break
                pc += 1 + (cnt + 1) // 2
        p = idx[int(kd.index_offset):int(kd.index_offset) + int(kd.num_index_rows) * n]
        c = cst[int(kd.constants_offset):int(kd.constants_offset) + int(kd.num_constant_rows) * n]
        pm.run_kernel(words, nl, x, p, c, n, int(kd.output_offset))
    assert planted
    ids = np.ascontiguousarray(w.out_index_data, np.uint32)
    s, n = int(d.output_start[0]), int(d.output_length[0])
    assert not np.array_equal(x[ids[s:s + n].astype(np.int64)], ref)


@pytest.mark.parametrize("seed", range(100, 116))
def test_random_plans_sweep(seed):
    """Sixteen more random expression plans (shapes, shared blocks, sizes)."""
    w = native.Workload("random", 500 + 97 * (seed % 7), seed)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    assert np.array_equal(model(w, w.inputs, native.MATH_EXACT).view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("name,size", [("cloth", 4), ("neohookean", 2)])
def test_literals_are_loaded_once(name, size):
    """The templates' distinct literals are loaded once each in the load
    section (in range of the literal table); no literal-load entries remain
    among the compute bundles."""
    w = native.Workload(name, size, 3)
    u = Created(w)
    seen = 0
    for k in range(w.plan.contents.num_kernels):
        for math_mode in (native.MATH_EXACT, native.MATH_FAST):
            words, _, nl = pm.kernel_program(u.lib, u.h, k, math_mode)
            w64 = [int(v) for v in words]
            pc = nl
            while w64[pc] & 0xff != pm.OP_END:
                assert w64[pc] & 0xff != pm.OP_LDK
                pc += 1 + (((w64[pc] >> 8) & 0xffff) + 1) // 2
            table = len(w64) - (pc + 1)
            lits = [v >> 32 for v in w64[:nl] if v & 0xff == pm.OP_LDK]
            assert len(lits) == len(set(lits)) and all(i < table for i in lits)
            seen += len(lits)
    assert seen > 0


def test_literals_beyond_the_load_section_cap():
    """A template with 40 distinct literals: the 32 most read are loaded in the
    load section, the other 8 stay literal-load entries; both modes agree with
    the oracle."""
    w = native.Workload("literals", 300, 3)
    u = Created(w)
    words, _, nl = pm.kernel_program(u.lib, u.h, 0, native.MATH_FAST)
    w64 = [int(v) for v in words]
    assert sum(1 for v in w64[:nl] if v & 0xff == pm.OP_LDK) == 32
    pc, entries = nl, 0
    while w64[pc] & 0xff != pm.OP_END:
        if w64[pc] & 0xff == pm.OP_LDK:
            entries += (w64[pc] >> 8) & 0xffff
        pc += 1 + (((w64[pc] >> 8) & 0xffff) + 1) // 2
    assert entries == 8
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    assert np.array_equal(model(w, w.inputs, native.MATH_EXACT).view(np.uint64), ref.view(np.uint64))
    assert rel_err(model(w, w.inputs, native.MATH_FAST), ref) <= 1e-12


@pytest.mark.parametrize("name,size", [("cotan", 12), ("cloth", 6), ("ata", 12), ("neohookean", 2), ("random", 3000),
                                       ("literals", 300)])
def test_program_format_invariants(name, size):
    """What the interpreter relies on, for every kernel in both modes: register
    numbers below the program's register count (the shared-memory register
    file is sized by it), no entry of a bundle reading or writing a register
    that another entry of the same bundle writes (entries run in any order
    across lanes), literal indices inside the literal table, accumulator flags
    only on single-entry bundles, and every output row of the kernel stored."""
    w = native.Workload(name, size, 5)
    u = Created(w)
    d = w.plan.contents
    for k in range(d.num_kernels):
        for math_mode in (native.MATH_EXACT, native.MATH_FAST):
            words, regs, nl = pm.kernel_program(u.lib, u.h, k, math_mode)
            w64 = [int(v) for v in words]
            pc = nl
            while w64[pc] & 0xff != pm.OP_END:
                pc += 1 + (((w64[pc] >> 8) & 0xffff) + 1) // 2
            table = len(w64) - (pc + 1)
            assert 0 < regs <= 255
            for v in w64[:nl]:
                op, dst, imm = v & 0xff, (v >> 8) & 0xff, v >> 32
                assert op in (pm.OP_LDX, pm.OP_LDC, pm.OP_LDK) and dst < regs
                if op == pm.OP_LDK:
                    assert imm < table
            stored = set()
            pc = nl
            while w64[pc] & 0xff != pm.OP_END:
                h = w64[pc]
                op, cnt, flags = h & 0xff, (h >> 8) & 0xffff, h & 0xff000000
                ents = [(w64[pc + 1 + q // 2] >> (32 * (q & 1))) & 0xffffffff for q in range(cnt)]
                pc += 1 + (cnt + 1) // 2
                assert cnt >= 1
                if flags & (pm.H_A_ACC | pm.H_B_ACC | pm.H_C_ACC | pm.H_NOSTORE):
                    assert cnt == 1
                if op == pm.OP_ST:
                    for e in ents:
                        assert (e & 0xff) < regs
                        stored.add(e >> 8)
                    continue
                if op == pm.OP_LDK:
                    assert all((e >> 8) < table for e in ents)
                    writes = [e & 0xff for e in ents]
                    reads = []
                else:
                    writes = [e & 0xff for e in ents]
                    reads = [(e >> (8 * (s + 1))) & 0xff for e in ents for s in range(pm.nsrc(op))
                             if not flags & (pm.H_A_ACC << s)]
                assert all(r < regs for r in writes + reads)
                if not flags & pm.H_NOSTORE:
                    assert len(set(writes)) == len(writes)
                    assert not set(writes) & set(reads)
            assert stored == set(range(d.kernels[k].num_output_rows))
