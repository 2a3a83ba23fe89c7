"""CPU tests: the oracle and the engine's front end against the reference's own
output (golden fixtures made by tests/golden/make_golden.sh from the reference
library built from its sources)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from symboliclib_gb300 import native

import oracle.cpu as ocpu


def split_inputs(w, flat):
    out, off = [], 0
    for a in w.inputs:
        out.append(flat[off:off + len(a)])
        off += len(a)
    return out


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_plan_equals_reference(name, size, seed):
    """Kernels, templates (operation order and exact constants), access tables,
    index / constant / output tables and memory size equal the reference's."""
    plan_ref, _, _ = load_golden(name, size)
    w = native.Workload(name, size, seed, 0, text=True)
    assert w.plan_text == plan_ref


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_inputs_are_the_golden_inputs(name, size, seed):
    _, inp, _ = load_golden(name, size)
    w = native.Workload(name, size, seed)
    for a, b in zip(split_inputs(w, inp), w.inputs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_oracle_bit_exact_vs_reference(name, size, seed):
    """The C oracle evaluates the reference's operation order: bit-identical to
    the reference ComputeUnit compiled without fast-math / FP contraction."""
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    out = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, split_inputs(w, inp))[0]
    assert out.shape == gold.shape
    assert np.array_equal(out.view(np.uint64), gold.view(np.uint64))


def rel_err(a, ref, floor_frac=1e-10):
    """Max |a - ref| / max(|ref|, floor), floor = floor_frac * max|ref|."""
    floor = floor_frac * np.max(np.abs(ref))
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor)))


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_numeric_model_vs_reference(name, size, seed):
    """The workload evaluated directly in double (the numeric FP64 oracle, the
    role Eigen's numeric expression plays in the reference's examples) agrees
    with the reference's symbolic evaluation to 1e-12 relative.  The two
    evaluate differently arranged formulas, so entries that are sums with
    cancellation (cloth Hessian couplings, whose terms are ~1e4 times larger
    than the sum) are compared against a floor of 1e-4 of the container's
    largest magnitude."""
    _, _, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    assert rel_err(w.numeric, gold, floor_frac=1e-4) <= 1e-12


def test_oracle_detects_a_changed_operation_order():
    """Planted fault, in the oracle only: reversing the operand order of one sum
    changes the result bits, so the bit-exact comparison has teeth."""
    name, size, seed = "cotan", 8, 22
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    d = w.plan.contents
    # find a kernel whose template has an n-ary ADD with >= 3 operands
    changed = False
    for k in range(d.num_kernels):
        kd = d.kernels[k]
        nodes = [kd.nodes[j] for j in range(kd.num_nodes)]
        if any(n.op == 3 and n.nchild >= 3 for n in nodes) and kd.num_instances > 1:
            # swap the first two index variables of the template
            idx = [j for j, n in enumerate(nodes) if n.op == 2 and n.b == -3]
            if len(idx) >= 2:
                a, b = kd.nodes[idx[0]].a, kd.nodes[idx[1]].a
                kd.nodes[idx[0]].a, kd.nodes[idx[1]].a = b, a
                changed = True
                break
    assert changed
    out = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, split_inputs(w, inp))[0]
    assert not np.array_equal(out.view(np.uint64), gold.view(np.uint64))


def test_vector_width_plan_shapes():
    """The CPU layout (vector width 4) pads kernels with more than 4 instances to
    a multiple of 4, as the reference's Kernel does (ComputeKernel.cpp:241-259)."""
    w0 = native.Workload("cotan", 8, 22, 0)
    w4 = native.Workload("cotan", 8, 22, 4)
    d0, d4 = w0.plan.contents, w4.plan.contents
    assert d0.num_kernels == d4.num_kernels
    for k in range(d0.num_kernels):
        n0, n4 = d0.kernels[k].num_instances, d4.kernels[k].num_instances
        if n0 > 4:
            assert n4 % 4 == 0 and n4 - n0 < 4
        else:
            assert n4 == n0


@pytest.mark.parametrize("seed", [22, 28, 3, 7])
def test_random_expression_plans_are_valid(seed):
    """Random expression DAGs, including seeds whose blocks collide on the
    reference's (GF(2)-linear) structure hash: the reference aborts on seed 22
    (ComputeKernel.cpp:166) and builds out-of-range index tables on seed 28;
    the engine splits such groups by structure, so every index stays inside x
    and the plan evaluates to the FP64 model."""
    w = native.Workload("random", 2000, seed)
    d = w.plan.contents
    for k in range(d.num_kernels):
        kd = d.kernels[k]
        n = kd.num_instances
        for a in range(kd.num_access):
            base, off = kd.access[2 * a], kd.access[2 * a + 1]
            p = w.index_data[kd.index_offset + base * n: kd.index_offset + (base + 1) * n].astype(np.int64) + off
            assert p.min() >= 0 and p.max() < d.num_total_memory
    out = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    assert rel_err(out, w.numeric) <= 1e-12
