"""Parity at the benchmark configurations, through the C ABI (GPU).

* cotan 500x500, one value set (the plain GPU path configuration): exact
  mode bit-identical to the CPU oracle with both executors and all three
  schedules; fast mode within 1e-12 per nonzero, entries below 1e-4 of the
  largest magnitude compared against that floor (the Laplacian's smallest
  entries come from cancelling products: there even the reference's own
  operation order is 4.8e-11 away from the FP64 numeric model).
* cloth 300x300 with 64 distinct value sets (the batched configuration):
  exact mode bit-identical to the oracle on sets 0, 31 and 63; fast mode
  within 1e-12 (floor 1e-4: the coupling entries are sums of terms up to 1e4
  times larger than the result).
* an uneven multi-pattern batch (cloth sides drawn log-uniform, 1 to 16 value
  sets each) in one graph replay: every unit bit-identical to the oracle.
* Neo-Hookean 10^3 cells: exact mode bit-identical to the oracle.
* the engine front end's tables equal the reference's own at cotan 500x500
  and cloth 200x200, in the CUDA and the CPU (VecWidth(4)) layouts (SHA-256
  digests recorded in tests/golden/reference_tables.json by
  tests/golden/make_table_hashes.py from the files the reference wrote);
* the reference's own generated CUDA, where oracle/ref_generate.sh kept it,
  built with --fmad=false: bit-identical to the engine's exact mode; its
  default build within the fast-mode tolerance.
The front end of the large workloads runs once per module."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT
from symboliclib_gb300 import native

import oracle.cpu as ocpu
from oracle import ref_paths

pytestmark = pytest.mark.gpu

SCHEDULES = [native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT]
EXECUTORS = [native.EXEC_COMPILED, native.EXEC_INTERPRETER]
TABLES = ROOT / "tests" / "golden" / "reference_tables.json"


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def rel_err(a, ref, floor_frac):
    floor = floor_frac * np.max(np.abs(ref))
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor)))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_tables(w, key):
    ref = json.loads(TABLES.read_text())[key]
    assert digest(w.index_data) == ref["indexData"]["sha256"], key
    assert digest(w.out_index_data) == ref["outIndexData"]["sha256"], key
    assert digest(w.const_data) == ref["constData"]["sha256"], key
    assert digest(np.concatenate(w.inputs)) == ref["inputs.bin"]["sha256"], key


@pytest.fixture(scope="module")
def cotan500():
    return native.Workload("cotan", 500, 2024)


@pytest.fixture(scope="module")
def cloth300():
    return native.Workload("cloth", 300, 2024)


@pytest.fixture(scope="module")
def cloth200():
    return native.Workload("cloth", 200, 2024)


@pytest.fixture(scope="module")
def cotan500_oracle(cotan500):
    w = cotan500
    return ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]


def test_cotan500_tables_equal_reference(cotan500):
    check_tables(cotan500, "cotan_500_cuda")


def test_cloth200_tables_equal_reference(cloth200):
    """cloth 200x200 is the largest cloth whose reference plan fits the 62 GB
    host the fixtures were generated on (the reference's front end needs more
    than that for 300x300)."""
    check_tables(cloth200, "cloth_200_cuda")


@pytest.mark.parametrize("name,size", [("cloth", 200), ("neohookean", 20)])
def test_reference_cpu_code_equals_oracle_at_size(name, size, tmp_path):
    """The reference CPU ComputeUnit's own generated code for cloth 200x200 and
    Neo-Hookean 20^3 (kept by oracle/ref_generate.sh), built in strict mode
    and run through its five calls, gives the oracle's results bit for bit
    (tests/test_reference_cpu_outputs.py does the smaller cases on any host;
    these run here, where the front end is fast)."""
    import os
    import shutil
    import subprocess
    if not ref_paths.available(name, size, "cpu"):
        pytest.skip("the reference's generated CPU code is not present here")
    gen = tmp_path / "gen"
    shutil.copytree(ref_paths.gen_dir(name, size, "cpu"), gen, ignore=shutil.ignore_patterns("*.so", "ref_run_cpu"))
    env = dict(os.environ, SYMREF_STRICT="1", NUMTHREADS="4")
    r = subprocess.run(["sh", str(ROOT / "oracle" / "ref_paths.sh"), str(gen), "cpu"], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    out = tmp_path / "results.bin"
    r = subprocess.run([str(gen / "ref_run_cpu"), str(gen), str(gen / "ref_cpu.so"), "0", "1", str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    ref = np.fromfile(out, np.float64)
    w = native.Workload(name, size, 2024)
    oracle = np.concatenate(ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs))
    assert bits_equal(ref, oracle)


@pytest.mark.parametrize("layout,width", [("cuda", 0), ("cpu", 4)])
def test_neohookean20_tables_equal_reference(layout, width):
    """The Neo-Hookean Hessian of a 20 x 20 x 20 cube (40,000 tets, 1,013,229
    nonzeros; the config-5 family at the largest size whose reference plan
    was made here) from the engine's front end, against the reference's
    tables in both layouts."""
    check_tables(native.Workload("neohookean", 20, 2024, vector_width=width), f"neohookean_20_{layout}")


@pytest.mark.parametrize("name,size", [("cotan", 500), ("cloth", 200)])
def test_cpu_layout_tables_equal_reference(name, size):
    """The reference CPU ComputeUnit's layout (VecWidth(4): padded, blocked
    tables) from the engine's front end, against the reference's own."""
    w = native.Workload(name, size, 2024, vector_width=4)
    check_tables(w, f"{name}_{size}_cpu")


@pytest.mark.parametrize("executor", EXECUTORS)
def test_cotan500_exact_bit_identical(cotan500, cotan500_oracle, executor):
    w = cotan500
    u = native.Unit.from_workload(w)
    u.set_arg(0, w.inputs[0])
    for kind in SCHEDULES:
        u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
        u.run()
        assert bits_equal(u.get_result(0), cotan500_oracle), kind


@pytest.mark.parametrize("executor", EXECUTORS)
def test_cotan500_fast_within_tolerance(cotan500, cotan500_oracle, executor):
    w = cotan500
    u = native.Unit.from_workload(w)
    u.set_arg(0, w.inputs[0])
    for kind in SCHEDULES:
        u.set_schedule(kind=kind, math=native.MATH_FAST, executor=executor)
        u.run()
        assert rel_err(u.get_result(0), cotan500_oracle, 1e-4) <= 1e-12, kind


def cloth_sets(w, S, seed=7):
    """S distinct states: the seeded positions moved by a small per-set field."""
    rng = np.random.default_rng(seed)
    X, V = w.inputs
    return [[X + 1e-3 * s * np.sin(np.arange(len(X)) * (0.01 + 0.001 * s)) + 1e-6 * rng.standard_normal(len(X)),
             V * (1.0 + 0.01 * s)] for s in range(S)]


@pytest.mark.parametrize("executor", EXECUTORS)
def test_cloth300_64_sets(cloth300, executor):
    w = cloth300
    S = 64
    sets = cloth_sets(w, S)
    u = native.Unit.from_workload(w)
    u.set_num_sets(S)
    for i in range(2):
        u.set_arg(i, np.concatenate([ps[i] for ps in sets]))
    refs = {s: ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, sets[s])[0] for s in (0, 31, 63)}
    kinds = SCHEDULES if executor == native.EXEC_COMPILED else [native.SCHEDULE_LEVELS]
    for kind in kinds:
        u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor, lanes_per_item=1)
        u.run()
        out = u.get_result(0).reshape(S, -1)
        for s, ref in refs.items():
            assert bits_equal(out[s], ref), (kind, s)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, executor=executor)
    u.run()
    out = u.get_result(0).reshape(S, -1)
    for s, ref in refs.items():
        assert rel_err(out[s], ref, 1e-4) <= 1e-12, s


def test_uneven_multi_pattern_batch():
    """Cloth patterns with sides drawn log-uniform from 8 to 64 and 1-16 value
    sets each, every unit with its own kernels and schedule, in one graph
    replay: each unit's first and last set bit-identical to the oracle."""
    import ctypes as C
    lib = native.symgb()
    rng = np.random.default_rng(2024)
    sides = np.unique(np.exp(rng.uniform(np.log(8), np.log(64), 24)).astype(int))
    units = []
    for k, side in enumerate(sides):
        w = native.Workload("cloth", int(side), 500 + int(side))
        u = native.Unit.from_workload(w)
        S = int(rng.integers(1, 17))
        u.set_schedule(kind=SCHEDULES[k % 3], math=native.MATH_EXACT, executor=EXECUTORS[k % 2])
        u.set_num_sets(S)
        per_set = [[a * (1.0 + 0.01 * s) for a in w.inputs] for s in range(S)]
        for i in range(2):
            u.set_arg(i, np.concatenate([ps[i] for ps in per_set]))
        ref = [ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, per_set[s])[0] for s in (0, S - 1)]
        units.append((w, u, S, ref))
    handles = (C.c_void_p * len(units))(*[u.handle.value for _, u, _, _ in units])
    b = C.c_void_p()
    native.check(lib.symgb_batch_create(handles, len(units), 8, C.byref(b)))
    try:
        for _ in range(2):
            native.check(lib.symgb_batch_run(b))
            for w, u, S, ref in units:
                out = u.get_result(0).reshape(S, -1)
                assert bits_equal(out[0], ref[0]) and bits_equal(out[S - 1], ref[1])
    finally:
        lib.symgb_batch_destroy(b)


def test_neohookean_10_exact():
    w = native.Workload("neohookean", 10, 2024)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    u = native.Unit.from_workload(w)
    u.set_arg(0, w.inputs[0])
    for executor in EXECUTORS:
        for kind in SCHEDULES:
            u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
            u.run()
            assert bits_equal(u.get_result(0), ref), (executor, kind)


def test_ata100_stated_size():
    """B = A^T A + A at its stated size (A 10,000 x 10,000: the 5-point stencil
    of a 100 x 100 grid plus 2 seeded random entries per column, 69,600
    nonzeros; B 365,700 nonzeros): exact mode bit-identical to the oracle in
    every schedule and executor, grouped items too; fast mode within 1e-12
    relative with the assembled matrices' floor of 1e-4 of the largest entry.
    B's smallest entries are sums that cancel (down to 5.6e-7 against a
    largest entry of 6.4), so FMA contraction moves them by a few units in the
    last place of their terms: 3.1e-17 absolute, 5.5e-11 relative at a 1e-10
    floor (the same fast-mode result as the host emulation of the generated
    code, which matches it bit for bit)."""
    w = native.Workload("ata", 100, 2024)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    u = native.Unit.from_workload(w)
    u.set_arg(0, w.inputs[0])
    for executor in EXECUTORS:
        for kind in SCHEDULES:
            u.set_schedule(kind=kind, math=native.MATH_EXACT, executor=executor)
            u.run()
            assert bits_equal(u.get_result(0), ref), (executor, kind)
            u.set_schedule(kind=kind, math=native.MATH_FAST, executor=executor)
            u.run()
            assert rel_err(u.get_result(0), ref, 1e-4) <= 1e-12, (executor, kind)
    u.set_item_layout(native.ITEMS_GROUPED)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT, items_per_thread=4)
    u.run()
    assert bits_equal(u.get_result(0), ref)


@pytest.mark.parametrize("name,size", [("cotan", 500), ("cloth", 200)])
def test_reference_generated_cuda_matches_engine(name, size, cotan500, cloth200, tmp_path):
    """The reference's generated CUDA for one value set, built by its own nvcc
    command with -arch=sm_103a --fmad=false, equals the engine's exact mode
    bit for bit; its default build (FMA contraction by nvcc) is within the
    fast-mode tolerance of it."""
    if not ref_paths.available(name, size, "cuda"):
        pytest.skip("the reference's generated code was not kept (oracle/ref_generate.sh)")
    w = cotan500 if name == "cotan" else cloth200
    res = ref_paths.gpu_paths(name, size, warmup=1, steps=3, results_dir=tmp_path)
    assert res["ref_exact"]["outputs"] == len(w.numeric)
    u = native.Unit.from_workload(w)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, a)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT)
    u.run()
    exact = u.get_result(0)
    ref_exact = np.fromfile(tmp_path / f"{name}_{size}_ref_exact.bin")
    assert bits_equal(ref_exact, exact)
    floor = 1e-4
    for lib in ("ref_default", "ref_sm103a"):
        got = np.fromfile(tmp_path / f"{name}_{size}_{lib}.bin")
        assert rel_err(got, exact, floor) <= 1e-12, lib
