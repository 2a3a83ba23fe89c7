"""Edge cases of the device path against the CPU oracle (exact mode,
bit-identical): the smallest meshes (kernels of one or two instances), a
template with more distinct literals than the load section takes,
random expression plans including groups split after structure-hash
collisions, subnormal and non-finite values, and a value-set count that is
no multiple of a warp; fast mode's division and square root across
magnitudes (within the fast-mode tolerance)."""
import numpy as np
import pytest

from symboliclib_gb300 import native

import oracle.cpu as ocpu

pytestmark = pytest.mark.gpu

SCHEDULES = [native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT]
EXECUTORS = [native.EXEC_COMPILED, native.EXEC_INTERPRETER]


def same_bits(a, b):
    """Bit-identical, treating every NaN as equal to every NaN."""
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(nan | (a.view(np.uint64) == b.view(np.uint64))))


def run_exact(w, inputs, kind, sets=1, executor=native.EXEC_COMPILED):
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
    u.set_num_sets(sets)
    for i, a in enumerate(inputs):
        u.set_arg(i, np.tile(a, sets))
    u.run()
    return u.get_result(0).reshape(sets, -1)


@pytest.mark.parametrize("name,size", [("cotan", 2), ("cotan", 3), ("cloth", 2), ("ata", 2), ("neohookean", 1),
                                       ("literals", 300)])
def test_smallest_meshes(name, size):
    w = native.Workload(name, size, 4)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    for executor in EXECUTORS:
        for kind in SCHEDULES:
            assert same_bits(run_exact(w, w.inputs, kind, executor=executor)[0], ref), (kind, executor)


@pytest.mark.parametrize("seed", [3, 22, 28, 41])
def test_random_expression_plans(seed):
    """Seeds 22 and 28 hold blocks whose CRC structure hashes collide; their
    groups are split by structure before kernel construction."""
    w = native.Workload("random", 20000, seed)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    for executor in EXECUTORS:
        for kind in SCHEDULES:
            assert same_bits(run_exact(w, w.inputs, kind, executor=executor)[0], ref), (kind, executor)


def test_subnormal_and_non_finite_values():
    w = native.Workload("cotan", 6, 2)
    x = w.inputs[0].copy()
    cases = {
        "subnormal products": x * 1e-160,
        "huge": x * 1e150,
        "inf and nan": np.where(np.arange(len(x)) % 17 == 3, np.inf, np.where(np.arange(len(x)) % 23 == 5, np.nan, x)),
        "zeros": np.where(np.arange(len(x)) % 5 == 0, 0.0, x),
    }
    for what, v in cases.items():
        ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, [v])[0]
        for executor in EXECUTORS:
            for kind in SCHEDULES:
                assert same_bits(run_exact(w, [v], kind, executor=executor)[0], ref), (what, kind, executor)


def test_fast_division_and_square_root_across_magnitudes():
    """Fast mode divides and takes square roots by refining the hardware
    approximation inside an exponent window and takes the IEEE operation
    outside it.  Random expression plans (quotients a / (b*b + 1), roots
    sqrt(a*a + b*b + 1)) on inputs outside the window, zero dividends of
    either sign, overflowing squares, inf and NaN: the same non-finite results
    as the oracle and the finite ones within the fast-mode tolerance."""
    for seed in (3, 41):
        w = native.Workload("random", 20000, seed)
        x = w.inputs[0]
        i = np.arange(len(x))
        rng = np.random.default_rng(seed)
        cases = {
            "tiny (outside the window)": x * 2.0 ** -520,
            "subnormal": x * 1e-310,
            "huge (squares overflow)": x * 1e200,
            "signed zeros": np.where(i % 5 == 0, 0.0, np.where(i % 7 == 0, -0.0, x)),
            "inf and nan": np.where(i % 17 == 3, -np.inf, np.where(i % 23 == 5, np.nan, x)),
            "mixed magnitudes": x * 10.0 ** rng.uniform(-300, 300, len(x)),
        }
        for what, v in cases.items():
            ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, [v])[0]
            u = native.Unit.from_workload(w)
            outs = []
            for executor in EXECUTORS:
                u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, executor=executor)
                u.set_arg(0, v)
                u.run()
                outs.append(u.get_result(0))
            assert same_bits(outs[0], outs[1]), (seed, what)  # the same operations in both executors
            out = outs[0]
            assert np.array_equal(np.isnan(out), np.isnan(ref)), (seed, what)
            assert np.array_equal(np.isinf(out), np.isinf(ref)), (seed, what)
            inf = np.isinf(ref)
            assert np.array_equal(np.sign(out[inf]), np.sign(ref[inf])), (seed, what)
            fin = np.isfinite(ref)
            if fin.any():
                a, r = out[fin], ref[fin]
                floor = max(1e-10 * np.max(np.abs(r)), np.finfo(float).tiny)
                assert np.max(np.abs(a - r) / np.maximum(np.abs(r), floor)) <= 1e-12, (seed, what)


def test_value_sets_not_a_multiple_of_a_warp():
    w = native.Workload("cloth", 4, 8)
    S = 257
    rng = np.random.default_rng(0)
    per_set = [[a * (1.0 + 0.01 * rng.standard_normal(a.shape)) for a in w.inputs] for _ in range(S)]
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
    u.set_num_sets(S)
    for i in range(len(w.inputs)):
        u.set_arg(i, np.concatenate([ps[i] for ps in per_set]))
    u.run()
    out = u.get_result(0).reshape(S, -1)
    for s in (0, 31, 32, 128, 256):
        ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, per_set[s])[0]
        assert same_bits(out[s], ref), s
