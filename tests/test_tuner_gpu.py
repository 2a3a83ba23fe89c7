"""GPU tests of schedules beyond the basic three, multi-unit graph batches,
the cost model's FP32 kernels (gradients against the CPU oracle) and the
learned schedule proposer."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from symboliclib_gb300 import native, tuner

import oracle.cpu as ocpu
import oracle.mlp as omlp

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def split_inputs(w, flat):
    out, off = [], 0
    for a in w.inputs:
        out.append(flat[off:off + len(a)])
        off += len(a)
    return out


@pytest.mark.parametrize("depth", [2, 3])
@pytest.mark.parametrize("graph", [0, 1])
def test_fusion_depth_and_graphs_bit_exact(depth, graph):
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 2, 42)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT, fusion_depth=depth, use_graph=graph,
                       executor=native.EXEC_INTERPRETER)
        for i, a in enumerate(split_inputs(w, inp)):
            u.set_arg(i, a)
        for _ in range(2):
            u.run()
            assert bits_equal(u.get_result(0), gold), (name, depth, graph)
        u.set_schedule(kind=native.SCHEDULE_PERSISTENT, math=native.MATH_EXACT, use_graph=graph,
                       executor=native.EXEC_INTERPRETER)
        u.run()
        assert bits_equal(u.get_result(0), gold), (name, "persistent", graph)


def test_every_tuner_schedule_is_exact():
    _, inp, gold = load_golden("cloth", 5)
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w)
    for i, a in enumerate(split_inputs(w, inp)):
        u.set_arg(i, a)
    for s in tuner.SPACE:
        s.apply(u, native.MATH_EXACT)
        u.run()
        assert bits_equal(u.get_result(0), gold), s


def test_batch_graph_matches_individual_runs():
    """Units of uneven size and value-set count in one graph replay."""
    lib = native.symgb()
    units, refs = [], []
    rng = np.random.default_rng(3)
    for k, (name, size) in enumerate([("cloth", 4), ("cloth", 9), ("cotan", 30), ("cloth", 6), ("ata", 10)]):
        w = native.Workload(name, size, 100 + k)
        u = native.Unit.from_workload(w)
        S = int(rng.integers(1, 17))
        kind = [native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT][k % 3]
        u.set_schedule(kind=kind, math=native.MATH_EXACT)
        u.set_num_sets(S)
        per_set = [[a * (1.0 + 0.01 * s) for a in w.inputs] for s in range(S)]
        for i in range(len(w.inputs)):
            u.set_arg(i, np.concatenate([ps[i] for ps in per_set]))
        ref = [ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, per_set[s])[0] for s in (0, S - 1)]
        units.append((w, u, S))
        refs.append(ref)
    handles = (C.c_void_p * len(units))(*[u.handle.value for _, u, _ in units])
    b = C.c_void_p()
    native.check(lib.symgb_batch_create(handles, len(units), 4, C.byref(b)))
    try:
        assert lib.symgb_batch_launch_count(b) >= len(units)
        for _ in range(2):
            native.check(lib.symgb_batch_run(b))
            for (w, u, S), ref in zip(units, refs):
                out = u.get_result(0).reshape(S, -1)
                assert bits_equal(out[0], ref[0]) and bits_equal(out[S - 1], ref[1])
    finally:
        lib.symgb_batch_destroy(b)


def test_mlp_gradient_matches_cpu_oracle():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((300, 23)).astype(np.float32)
    y = rng.standard_normal(300).astype(np.float32)
    net = native.MLP(23, 64, seed=5)
    g, loss = net.gradient(X, y)
    g_ref, loss_ref = omlp.gradient(net.params(), X, y, 23, 64)
    assert abs(loss - loss_ref) <= 1e-4 * max(1.0, loss_ref)
    scale = np.max(np.abs(g_ref))
    assert np.max(np.abs(g - g_ref)) <= 1e-4 * scale
    pred = net.predict(X)
    ref_pred, _ = omlp.forward(net.params(), X, 23, 64)
    assert np.max(np.abs(pred - ref_pred)) <= 1e-4 * max(1.0, np.max(np.abs(ref_pred)))


def test_mlp_training_fits_a_smooth_function():
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (2000, 4)).astype(np.float32)
    y = (np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] - 0.5 * X[:, 3] ** 2).astype(np.float32)
    net = native.MLP(4, 64, seed=2)
    before = float(np.mean((net.predict(X) - y) ** 2))
    after = net.train(X, y, epochs=2000, lr=3e-3)
    assert after < 0.05 * before and after < 0.01


def test_learned_proposer_gain():
    """What the trained network gains, measured honestly.  The cost model is
    trained on the tuner's own exhaustive timings of one set of units and
    evaluated on held-out units (cotangent Laplacians and cloth Hessians of
    other sizes, one and eight value sets, random expression plans).  With the
    network, tuning times the default schedule plus the model's K - 1
    best-ranked others; without it, the default plus K - 1 others drawn at
    random.  K is at least 10x smaller than the schedule space.  Mean regret
    against exhaustive search must be at most 5% and no worse than without
    the network."""
    K = len(tuner.SPACE) // 15
    train_units = [("random", 60000, s, 1) for s in range(6)] + [("cotan", 100, 1, 1), ("cloth", 20, 2, 1),
                                                                  ("cloth", 12, 3, 8), ("ata", 60, 3, 1)]
    test_units = [("random", 90000, 100 + s, 1) for s in range(2)] + [("cotan", 150, 7, 1), ("cotan", 220, 8, 1),
                                                                     ("cloth", 26, 8, 1), ("cloth", 16, 9, 8)]
    X, y, held = [], [], []
    for spec in train_units + test_units:
        name, size, seed, S = spec
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        u.set_num_sets(S)
        for i, a in enumerate(w.inputs):
            u.set_arg(i, np.tile(a, S))
        stream = tuner.bind_stream(u)
        res = tuner.exhaustive(u, stream, runs=5)
        st = u.stats()
        if spec in train_units:
            for sch, t in res.timings.items():
                X.append(tuner.features(st, S, sch))
                y.append(t)
        else:
            held.append((res, st, S))
    model = tuner.CostModel(seed=0)
    model.fit(np.stack(X), np.array(y), epochs=3000)
    rng = np.random.default_rng(4)
    regret_model, regret_blind, regret_default = [], [], []
    others = [sch for sch in tuner.SPACE if sch != tuner.DEFAULT]
    for res, st, S in held:
        picks = tuner.propose(model, st, S, k=K)
        assert len(picks) == K and picks[0] == tuner.DEFAULT
        regret_model.append(min(res.timings[sch] for sch in picks if sch in res.timings) / res.best_us - 1.0)
        regret_default.append(res.timings[tuner.DEFAULT] / res.best_us - 1.0)
        for _ in range(50):  # expected regret of the default plus K - 1 random picks
            blind = [tuner.DEFAULT] + [others[i] for i in rng.choice(len(others), K - 1, replace=False)]
            regret_blind.append(min(res.timings[sch] for sch in blind if sch in res.timings) / res.best_us - 1.0)
    print(f"mean regret: default {np.mean(regret_default):.4f}, default + {K - 1} random "
          f"{np.mean(regret_blind):.4f}, default + model's top {K - 1} {np.mean(regret_model):.4f}")
    assert len(tuner.SPACE) / K >= 10
    assert np.mean(regret_model) <= 0.05
    assert np.mean(regret_model) <= np.mean(regret_blind)


def test_per_kernel_shapes_are_exact_and_timed():
    """Per-kernel launch shapes (plain and levels schedules) change no value;
    per-kernel timing returns one positive time per launched kernel."""
    torch = pytest.importorskip("torch")
    for name, size, seed in [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 2, 42)]:
        _, inp, gold = load_golden(name, size)
        w = native.Workload(name, size, seed)
        u = native.Unit.from_workload(w)
        for i, a in enumerate(split_inputs(w, inp)):
            u.set_arg(i, a)
        rng = np.random.default_rng(seed)
        for trial in range(3):
            for k in range(u.num_kernels):
                i, l, t = tuner.KERNEL_SHAPES[rng.integers(len(tuner.KERNEL_SHAPES))]
                u.set_kernel_shape(k, i, l, t)
            for kind in (native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS):
                for executor in (native.EXEC_COMPILED, native.EXEC_INTERPRETER):
                    u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
                    u.run()
                    assert bits_equal(u.get_result(0), gold), (name, trial, kind, executor)
        flush = torch.empty(1 << 20, dtype=torch.float32, device="cuda")
        t = u.time_kernels(3, flush)
        assert len(t) == u.num_kernels
        assert all(t[k] > 0 for k in range(u.num_kernels) if u.kernel_instances[k])
        u.run()
        assert bits_equal(u.get_result(0), gold)


def test_per_kernel_tuning_picks_the_fastest_shape():
    """tune_kernels keeps, per kernel, the shape of least time, and the learned
    per-kernel proposer (trained on other units) lands within 10% of it."""
    X, y = [], []
    for spec in [("cloth", 10, 3), ("cotan", 60, 4), ("random", 40000, 5)]:
        w = native.Workload(*spec)
        u = native.Unit.from_workload(w)
        for i, a in enumerate(w.inputs):
            u.set_arg(i, a)
        res = tuner.tune_kernels(u, reps=3)
        sums = [tuner.program_summary(u, k) for k in range(u.num_kernels)]
        for sh, t in res.table.items():
            for k in range(u.num_kernels):
                if u.kernel_instances[k] and t[k] > 0:
                    X.append(tuner.kernel_features(u, k, 1, sh, sums[k]))
                    y.append(t[k])
    model = tuner.KernelCostModel(seed=1)
    model.fit(np.stack(X), np.array(y), epochs=2000)
    w = native.Workload("cloth", 14, 9)
    u = native.Unit.from_workload(w)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, a)
    full = tuner.tune_kernels(u, reps=3)
    for k in range(u.num_kernels):
        if u.kernel_instances[k]:
            assert full.us[k] == min(full.table[sh][k] for sh in full.table)
    learned = tuner.tune_kernels_with_model(u, model, 1, k_top=2, reps=3)
    total = sum(full.table[sh][k] for k, sh in enumerate(learned.shapes))
    print("per-kernel regret", total / full.total_us - 1.0)
    assert total <= 1.10 * full.total_us
