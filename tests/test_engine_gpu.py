"""GPU parity tests: the CUDA engine, called through the C ABI, against the
reference's own results (golden fixtures) and the CPU oracle.

Exact mode must be bit-identical for every schedule and batch size; fast mode
(FMA contraction) must agree to 1e-12 relative per nonzero, entries below a
floor compared against that floor: 1e-10 of the container's largest magnitude,
and 1e-4 for the assembled matrices (cotangent Laplacian, cloth and
Neo-Hookean Hessians), whose small entries are sums of terms up to ~1e4 times
larger than the result (contraction rounds those terms
differently; an exact emulation of the FMA program gives the same error)."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from symboliclib_gb300 import native

import oracle.cpu as ocpu

pytestmark = pytest.mark.gpu

SCHEDULES = [native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT]
EXECUTORS = [native.EXEC_COMPILED, native.EXEC_INTERPRETER]
TOL = 1e-12
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


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
@pytest.mark.parametrize("kind", SCHEDULES)
@pytest.mark.parametrize("executor", EXECUTORS)
def test_exact_mode_bit_identical_to_reference(name, size, seed, kind, executor):
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
    for i, a in enumerate(split_inputs(w, inp)):
        u.set_arg(i, a)
    u.run()
    assert bits_equal(u.get_result(0), gold)


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
@pytest.mark.parametrize("kind", SCHEDULES)
@pytest.mark.parametrize("executor", EXECUTORS)
def test_fast_mode_within_tolerance(name, size, seed, kind, executor):
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=kind, math=native.MATH_FAST, executor=executor)
    for i, a in enumerate(split_inputs(w, inp)):
        u.set_arg(i, a)
    u.run()
    assert rel_err(u.get_result(0), gold, FAST_FLOOR.get(name, 1e-10)) <= TOL


@pytest.mark.parametrize("name,size,seed", [("cotan", 8, 22), ("cloth", 5, 32), ("ata", 9, 12)])
@pytest.mark.parametrize("kind", SCHEDULES)
@pytest.mark.parametrize("sets", [2, 7, 8, 32, 33, 64])
@pytest.mark.parametrize("executor", EXECUTORS)
def test_value_set_batches_match_oracle(name, size, seed, kind, sets, executor):
    """S value sets in one run: every set bit-identical (exact mode) to the
    oracle evaluated on that set alone."""
    w = native.Workload(name, size, seed)
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
    u.set_num_sets(sets)
    rng = np.random.default_rng(seed + sets)
    per_set = [[a * (1.0 + 0.05 * rng.standard_normal(a.shape)) for a in w.inputs] for _ in range(sets)]
    for i in range(len(w.inputs)):
        u.set_arg(i, np.concatenate([ps[i] for ps in per_set]))
    u.run()
    out = u.get_result(0).reshape(sets, -1)
    for s in (0, sets // 2, sets - 1):
        ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, per_set[s])[0]
        assert bits_equal(out[s], ref), f"set {s}"


@pytest.mark.parametrize("kind", SCHEDULES)
@pytest.mark.parametrize("executor", EXECUTORS)
def test_graph_replay_matches(kind, executor):
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=kind, math=native.MATH_EXACT, use_graph=1, executor=executor)
    for i, a in enumerate(split_inputs(w, inp)):
        u.set_arg(i, a)
    for _ in range(3):
        u.run()
        assert bits_equal(u.get_result(0), gold)
    assert u.last_launch_count() > 0


@pytest.mark.parametrize("tpb", [32, 64, 256])
@pytest.mark.parametrize("items", [1, 2, 4])
def test_block_sizes_and_items_per_thread(tpb, items):
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        for kind in SCHEDULES:
            for tile in (0, 3 * tpb):
                u.set_schedule(kind=kind, math=native.MATH_EXACT, threads_per_block=tpb, items_per_tile=tile,
                               items_per_thread=items, executor=native.EXEC_INTERPRETER)
                for i, a in enumerate(split_inputs(w, inp)):
                    u.set_arg(i, a)
                u.run()
                assert bits_equal(u.get_result(0), gold), (name, kind, tile)


@pytest.mark.parametrize("lanes", [2, 4, 8])
@pytest.mark.parametrize("tpb", [32, 128])
def test_lanes_per_item(lanes, tpb):
    """Several threads per work item split its bundles: results unchanged, for
    every schedule, partial tiles and several value sets."""
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 2, 42)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        for kind in SCHEDULES:
            for tile in (0, 3 * tpb // lanes + 1):
                u.set_schedule(kind=kind, math=native.MATH_EXACT, threads_per_block=tpb, items_per_tile=tile,
                               lanes_per_item=lanes, executor=native.EXEC_INTERPRETER)
                u.set_num_sets(1)
                for i, a in enumerate(split_inputs(w, inp)):
                    u.set_arg(i, a)
                u.run()
                assert bits_equal(u.get_result(0), gold), (name, kind, tile)
        u.set_num_sets(5)
        for i, a in enumerate(split_inputs(w, inp)):
            u.set_arg(i, np.tile(a, 5))
        u.run()
        out = u.get_result(0).reshape(5, -1)
        assert bits_equal(out[0], gold) and bits_equal(out[4], gold), name


@pytest.mark.parametrize("sets", [1, 3, 40])
def test_results_into_page_locked_memory(sets):
    """getResult into page-locked host memory (written by the gather kernel
    directly) equals getResult into ordinary memory."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
    u.set_num_sets(sets)
    for i, a in enumerate(split_inputs(w, inp)):
        u.set_arg(i, np.tile(a, sets))
    u.run()
    ordinary = u.get_result(0)
    pinned = torch.full((len(gold) * sets,), -1.0, dtype=torch.float64).pin_memory()
    native.check(native.symgb().symgb_get_result_sets(u.handle, C.c_void_p(pinned.data_ptr()), 0))
    assert bits_equal(pinned.numpy(), ordinary)
    assert bits_equal(pinned.numpy()[:len(gold)], gold)


def test_async_transfers_between_two_units():
    """Two units of one plan on two streams, fed and read with the async
    page-locked calls in alternation (the pipelined end-to-end pattern):
    every step's results equal the golden ones; pageable memory is refused."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    lib = native.symgb()
    units = []
    for _ in range(2):
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
        st = torch.cuda.Stream()
        native.check(lib.symgb_set_stream(u.handle, C.c_void_p(st.cuda_stream)))
        ins = [torch.from_numpy(a.copy()).pin_memory() for a in split_inputs(w, inp)]
        outs = [torch.full((len(gold),), -1.0, dtype=torch.float64).pin_memory() for _ in range(3)]
        units.append((u, st, ins, outs))
    for k in range(6):
        u, st, ins, outs = units[k % 2]
        for i, a in enumerate(ins):
            native.check(lib.symgb_set_arg_sets_async(u.handle, C.c_void_p(a.data_ptr()), i))
        native.check(lib.symgb_run_async(u.handle))
        native.check(lib.symgb_get_result_sets_async(u.handle, C.c_void_p(outs[k // 2].data_ptr()), 0))
    for u, _, _, outs in units:
        native.check(lib.symgb_synchronize(u.handle))
        for o in outs:
            assert bits_equal(o.numpy(), gold)
    page = np.empty(len(gold))
    assert lib.symgb_get_result_sets_async(units[0][0].handle, page.ctypes.data, 0) == -1


def test_async_results_of_consecutive_executes_stay_apart():
    """The async result copy runs on the unit's copy stream while the unit's
    stream goes on: with different inputs in every step, 2 then 3 value sets,
    and one destination per step, every destination holds its own step's
    results (exact mode, bit-identical to the oracle)."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    w = native.Workload("cloth", 6, 5)
    lib = native.symgb()
    rng = np.random.default_rng(11)
    units = []
    for _ in range(2):
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
        st = torch.cuda.Stream()
        native.check(lib.symgb_set_stream(u.handle, C.c_void_p(st.cuda_stream)))
        units.append(u)
    nnz = len(w.numeric)
    for sets in (2, 3):
        for u in units:
            u.set_num_sets(sets)
        steps = []
        for k in range(8):
            per_set = [[a * (1.0 + 0.05 * rng.standard_normal(a.shape)) for a in w.inputs] for _ in range(sets)]
            ins = [torch.from_numpy(np.concatenate([ps[i] for ps in per_set])).pin_memory()
                   for i in range(len(w.inputs))]
            out = torch.full((nnz * sets,), -1.0, dtype=torch.float64).pin_memory()
            u = units[k % 2]
            for i, a in enumerate(ins):
                native.check(lib.symgb_set_arg_sets_async(u.handle, C.c_void_p(a.data_ptr()), i))
            native.check(lib.symgb_run_async(u.handle))
            native.check(lib.symgb_get_result_sets_async(u.handle, C.c_void_p(out.data_ptr()), 0))
            steps.append((per_set, ins, out))
        for u in units:
            native.check(lib.symgb_synchronize(u.handle))
        for per_set, _, out in steps:
            got = out.numpy().reshape(sets, -1)
            for s in range(sets):
                ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, per_set[s])[0]
                assert bits_equal(got[s], ref), (sets, s)


@pytest.mark.parametrize("copy_streams", [1, 3, 8])
def test_async_result_copy_in_chunks(copy_streams):
    """A 72 MiB result (cloth 60 x 60, 64 value sets) split over up to 8 copy
    streams arrives whole: bit-identical to the synchronous result, twice in a
    row (the second gather waits for every chunk of the first copy)."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    w = native.Workload("cloth", 60, 4)
    lib = native.symgb()
    sets = 64
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
    u.set_num_sets(sets)
    u.set_copy_streams(copy_streams)
    ins = [torch.from_numpy(np.tile(a, sets)).pin_memory() for a in w.inputs]
    for i, a in enumerate(ins):
        native.check(lib.symgb_set_arg_sets(u.handle, C.c_void_p(a.data_ptr()), i))
    u.run()
    ref = u.get_result(0)
    assert len(ref) * 8 >= 8 * (8 << 20)
    outs = [torch.full((len(ref),), -1.0, dtype=torch.float64).pin_memory() for _ in range(2)]
    for o in outs:
        native.check(lib.symgb_run_async(u.handle))
        native.check(lib.symgb_get_result_sets_async(u.handle, C.c_void_p(o.data_ptr()), 0))
    native.check(lib.symgb_synchronize(u.handle))
    for o in outs:
        assert bits_equal(o.numpy(), ref)
    assert lib.symgb_set_copy_streams(u.handle, 0) == -1 and lib.symgb_set_copy_streams(u.handle, 9) == -1


def test_larger_cases_match_oracle():
    """Sizes beyond the fixtures: engine exact mode vs the CPU oracle."""
    for name, size, seed in [("cotan", 60, 5), ("ata", 30, 6), ("cloth", 12, 7)]:
        w = native.Workload(name, size, seed)
        ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
        assert rel_err(w.numeric, ref, floor_frac=1e-4) <= TOL
        u = native.Unit.from_workload(w)
        for executor in EXECUTORS:
            for kind in SCHEDULES:
                u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
                for i, a in enumerate(w.inputs):
                    u.set_arg(i, a)
                u.run()
                assert bits_equal(u.get_result(0), ref), (name, kind, executor)


@pytest.mark.parametrize("tpb,items,minb", [(32, 1, 0), (96, 2, 0), (128, 4, 0), (256, 1, 0), (512, 2, 0),
                                            (64, 4, 6), (128, 2, 8)])
@pytest.mark.parametrize("kind", SCHEDULES)
def test_compiled_block_sizes(tpb, items, minb, kind):
    """The compiled executor at several block sizes, work items per thread and
    register caps (minimum resident CTAs per SM), with partial last blocks,
    level dispatch boundaries and 1 or 5 value sets: bit-identical."""
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 1, 41)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=kind, math=native.MATH_EXACT, threads_per_block=tpb, items_per_thread=items,
                       blocks_per_sm=minb)
        for sets in (1, 5):
            u.set_num_sets(sets)
            for i, a in enumerate(split_inputs(w, inp)):
                u.set_arg(i, np.tile(a, sets))
            u.run()
            out = u.get_result(0).reshape(sets, -1)
            assert bits_equal(out[0], gold) and bits_equal(out[-1], gold), (name, sets)


def test_compiled_and_interpreted_per_kernel_shapes():
    """Per-kernel block sizes (plain launches of the compiled executor) and
    per-kernel timing work with both executors; values unchanged."""
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w)
    for k in range(u.num_kernels):
        u.set_kernel_shape(k, items=1 + (k % 2), lanes=1, tpb=32 * (1 + k % 4))
    for executor in EXECUTORS:
        u.set_schedule(kind=native.SCHEDULE_PLAIN, math=native.MATH_EXACT, executor=executor)
        for i, a in enumerate(split_inputs(w, inp)):
            u.set_arg(i, a)
        u.run()
        assert bits_equal(u.get_result(0), gold)
        us = u.time_kernels(reps=2)
        assert us.shape == (u.num_kernels,) and np.all(us >= 0)
        u.run()
        assert bits_equal(u.get_result(0), gold)


@pytest.mark.parametrize("path", [native.LOAD_READONLY, native.LOAD_L1, native.LOAD_L2])
@pytest.mark.parametrize("kind", SCHEDULES)
def test_compiled_load_paths(path, kind):
    """Every load data path of the compiled executor gives the reference's
    results bit for bit (1 and 33 value sets)."""
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 1, 41)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=kind, math=native.MATH_EXACT, items_per_thread=2)
        u.set_load_path(path)
        for sets in (1, 33):
            u.set_num_sets(sets)
            for i, a in enumerate(split_inputs(w, inp)):
                u.set_arg(i, np.tile(a, sets))
            u.run()
            out = u.get_result(0).reshape(sets, -1)
            assert bits_equal(out[0], gold) and bits_equal(out[-1], gold), (name, sets)


@pytest.mark.parametrize("items", [1, 2, 4])
@pytest.mark.parametrize("kind", SCHEDULES)
def test_compiled_grouped_items(items, kind):
    """The grouped item layout (consecutive instances per thread, vector loads
    from padded table copies) gives the reference's results bit for bit with 1
    and 64 value sets (5 for Neo-Hookean, whose modules compile slowly), and
    switching layouts back and forth keeps them."""
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 1, 41), ("ata", 9, 12)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        for layout in (native.ITEMS_GROUPED, native.ITEMS_STRIDED, native.ITEMS_GROUPED):
            u.set_item_layout(layout)
            u.set_schedule(kind=kind, math=native.MATH_EXACT, threads_per_block=64, items_per_thread=items)
            for sets in ((5,) if name == "neohookean" else (1, 64)):
                u.set_num_sets(sets)
                for i, a in enumerate(split_inputs(w, inp)):
                    u.set_arg(i, np.tile(a, sets))
                u.run()
                out = u.get_result(0).reshape(sets, -1)
                assert bits_equal(out[0], gold) and bits_equal(out[-1], gold), (name, layout, sets)


def test_grouped_items_at_larger_sizes_match_oracle():
    """Grouped layout on plans beyond the fixtures (partial last groups of
    every size), exact mode against the CPU oracle."""
    for name, size, seed in [("cotan", 61, 5), ("cloth", 13, 7), ("random", 30001, 3)]:
        w = native.Workload(name, size, seed)
        ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
        u = native.Unit.from_workload(w)
        u.set_item_layout(native.ITEMS_GROUPED)
        for items in (2, 4):
            for kind in SCHEDULES:
                u.set_schedule(kind=kind, math=native.MATH_EXACT, threads_per_block=128, items_per_thread=items)
                for i, a in enumerate(w.inputs):
                    u.set_arg(i, a)
                u.run()
                assert bits_equal(u.get_result(0), ref), (name, items, kind)


def duplicated_output_plan(w, count=10):
    """The workload's plan with a second output container that repeats the
    first `count` results (their slots then name two result positions, so
    their rows cannot be written straight into the result buffer)."""
    d = w.plan.contents
    n0 = int(d.output_length[0])
    desc = native.PlanDesc()
    for name, _ in native.PlanDesc._fields_:
        setattr(desc, name, getattr(d, name))
    starts = (C.c_uint64 * 2)(0, n0)
    lengths = (C.c_uint64 * 2)(n0, count)
    desc.num_outputs, desc.output_start, desc.output_length = 2, starts, lengths
    desc.num_output_values = n0 + count
    ids = np.concatenate([w.out_index_data[:n0], w.out_index_data[:count]]).astype(np.uint32)
    return desc, (starts, lengths), ids



@pytest.mark.parametrize("kind", SCHEDULES)
def test_direct_outputs_match_the_gathered_results(kind):
    """Results written straight at their positions (the default with the
    compiled executor and one value set) equal the gathered ones bit for bit,
    through every read path: host, page-locked, device and asynchronous."""
    torch = pytest.importorskip("torch")
    lib = native.symgb()
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 1, 41), ("ata", 9, 12)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=kind, math=native.MATH_EXACT)
        for i, a in enumerate(split_inputs(w, inp)):
            u.set_arg(i, a)
        for direct in (False, True):
            u.set_direct_outputs(direct)
            u.run()
            assert bits_equal(u.get_result(0), gold), (name, direct)
            pinned = torch.full((len(gold),), -1.0, dtype=torch.float64).pin_memory()
            native.check(lib.symgb_get_result_sets(u.handle, C.c_void_p(pinned.data_ptr()), 0))
            assert bits_equal(pinned.numpy(), gold), (name, direct)
            dev = torch.full((len(gold),), -1.0, dtype=torch.float64, device="cuda")
            native.check(lib.symgb_get_result_sets_device(u.handle, C.c_void_p(dev.data_ptr()), 0))
            native.check(lib.symgb_synchronize(u.handle))
            assert bits_equal(dev.cpu().numpy(), gold), (name, direct)
            outs = [torch.full((len(gold),), -1.0, dtype=torch.float64).pin_memory() for _ in range(3)]
            for o in outs:
                native.check(lib.symgb_run_async(u.handle))
                native.check(lib.symgb_get_result_sets_async(u.handle, C.c_void_p(o.data_ptr()), 0))
            native.check(lib.symgb_synchronize(u.handle))
            for o in outs:
                assert bits_equal(o.numpy(), gold), (name, direct)


def test_direct_outputs_with_shared_result_slots():
    """A plan whose second output container repeats results of the first: the
    rows holding the shared slots are gathered into the result buffer, the
    others written straight; both containers come out right, also after a
    graph replay and with an interpreter run in between."""
    _, inp, gold = load_golden("cotan", 8)
    w = native.Workload("cotan", 8, 22)
    desc, keep, ids = duplicated_output_plan(w)
    u = native.Unit(C.pointer(desc), w.index_data, ids, w.const_data)
    for executor, graph in ((native.EXEC_COMPILED, 0), (native.EXEC_INTERPRETER, 0), (native.EXEC_COMPILED, 1)):
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT, executor=executor, use_graph=graph)
        for i, a in enumerate(split_inputs(w, inp)):
            u.set_arg(i, a)
        u.run()
        assert bits_equal(u.get_result(0), gold), (executor, graph)
        assert bits_equal(u.get_result(1), gold[:10]), (executor, graph)
