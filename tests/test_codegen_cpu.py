"""The compiled executor's code generator on the CPU.

The module the engine generates for NVRTC is checked twice without a GPU:
  * NVRTC compiles it for sm_103a (every schedule kind, both math modes);
  * its kernel bodies, cut out of the module and compiled on the host by g++
    against a small header that maps the CUDA intrinsics onto IEEE host
    arithmetic (no contraction), are run over every instance in plan order:
    exact mode must reproduce the reference's golden results bit for bit, and
    the CPU oracle's on larger plans; fast mode (its division and square root
    replaced by the IEEE operations, within one unit in the last place of the
    device's) must stay within the fast-mode tolerance.
Units are only created, never initialised."""
import ctypes as C
import hashlib
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden
from symboliclib_gb300 import native

import oracle.cpu as ocpu

BUILD = ROOT / "symboliclib_gb300" / "_build" / "codegen_tests"
FAST_FLOOR = {"cloth": 1e-4, "neohookean": 1e-4, "cotan": 1e-4}

HOST_SHIM = r"""
#include <cmath>
#include <cstring>
#define __device__
#define __forceinline__ inline
#define SYMGB_XR __restrict__
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __ddiv_rn(double a, double b) { return a / b; }
static inline double __dsqrt_rn(double a) { return std::sqrt(a); }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
static inline double __longlong_as_double(long long v) { double d; std::memcpy(&d, &v, 8); return d; }
static inline double symgbNegate(double x) { return -x; }
static inline double symgbFastDiv(double a, double b) { return a / b; }
static inline double symgbFastRec(double x) { return 1.0 / x; }
static inline double symgbFastSqrt(double x) { return std::sqrt(x); }
template <class T> static inline T __ldg(const T* p) { return *p; }
#define SYMGB_LD(a) (*(a))
template <int IT> static inline void symgbLoadIdx(const unsigned* a, unsigned (&q)[IT]) {
    for (int j = 0; j < IT; ++j) q[j] = a[j];
}
template <int IT> static inline void symgbLoadConst(const double* a, double (&v)[IT]) {
    for (int j = 0; j < IT; ++j) v[j] = a[j];
}
template <int L2> static inline double symgbLoadX(const double* a) { return *a; }
"""


def host_library(source: str, num_kernels: int) -> C.CDLL:
    """Compiles the kernel bodies of a generated module for the host."""
    start = source.index("// kernel 0:")
    end = source.index('extern "C"')
    bodies = source[start:end]
    driver = ['extern "C" void symgb_host_run(int k, const double* x, double* xw, const unsigned* p, '
              'const double* c, unsigned long long n, unsigned S) {',
              "    for (unsigned long long i = 0; i < n; ++i)", "        for (unsigned s = 0; s < S; ++s)",
              "            switch (k) {"]
    for k in range(num_kernels):
        if f"symgbBody{k}(" in bodies:
            driver.append(f"                case {k}: symgbBody{k}<0>(x, xw, p, c, nullptr, nullptr, i, s); break;")
    driver += ["                default: break;", "            }", "}"]
    text = HOST_SHIM + bodies + "\n".join(driver) + "\n"
    BUILD.mkdir(parents=True, exist_ok=True)
    tag = hashlib.sha1(text.encode()).hexdigest()[:16]
    src, lib = BUILD / f"m_{tag}.cpp", BUILD / f"m_{tag}.so"
    if not lib.exists():
        src.write_text(text)
        subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                        str(src), "-o", str(lib)], check=True, capture_output=True)
    h = C.CDLL(str(lib))
    h.symgb_host_run.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint]
    return h


def run_generated(w, inputs, math, S=1):
    """Evaluates a workload's plan with its generated kernel bodies on the host
    (value sets laid out [slot][set] as on the device).  Returns output
    container 0 as [S][len]."""
    u = native.Unit.from_workload(w, init=False)
    u.set_schedule(kind=native.SCHEDULE_PLAIN, math=math)
    u.set_num_sets(S)
    src = u.compiled_source(native.SCHEDULE_PLAIN)
    d = w.plan.contents
    lib = host_library(src, d.num_kernels)
    x = np.zeros(int(d.num_total_memory) * S)
    for i, a in enumerate(inputs):
        start = int(d.arg_start[i])
        per_set = np.asarray(a).reshape(S, -1)
        for s in range(S):
            x[(start + np.arange(per_set.shape[1])) * S + s] = per_set[s]
    p = np.ascontiguousarray(w.index_data, np.uint32)
    c = np.ascontiguousarray(w.const_data, np.float64)
    if not len(p):
        p = np.zeros(1, np.uint32)
    if not len(c):
        c = np.zeros(1)
    for k in range(d.num_kernels):
        lib.symgb_host_run(k, x.ctypes.data, x.ctypes.data, p.ctypes.data, c.ctypes.data,
                           int(d.kernels[k].num_instances), S)
    ids = np.asarray(w.out_index_data[int(d.output_start[0]):int(d.output_start[0]) + int(d.output_length[0])],
                     np.int64)
    return np.stack([x[ids * S + s] for s in range(S)])


def grouped_host_library(source: str, num_kernels: int, items: int) -> C.CDLL:
    """The grouped-layout bodies (symgbGroup<k>) of a generated module, for the host."""
    start = source.index("// kernel 0:")
    end = source.index('extern "C"')
    bodies = source[start:end]
    driver = ['extern "C" void symgb_host_group(int k, const double* x, double* xw, const unsigned* p, '
              'const double* c, unsigned long long groups, unsigned S) {',
              "    for (unsigned long long g = 0; g < groups; ++g)", "        for (unsigned s = 0; s < S; ++s)",
              "            switch (k) {"]
    for k in range(num_kernels):
        if f"symgbGroup{k}(" in bodies:
            driver.append(f"                case {k}: symgbGroup{k}<0, {items}, false>(x, xw, p, c, nullptr, nullptr, g, s);"
                          " break;")
    driver += ["                default: break;", "            }", "}"]
    text = HOST_SHIM + bodies + "\n".join(driver) + "\n"
    BUILD.mkdir(parents=True, exist_ok=True)
    tag = hashlib.sha1(text.encode()).hexdigest()[:16]
    src, lib = BUILD / f"g_{tag}.cpp", BUILD / f"g_{tag}.so"
    if not lib.exists():
        src.write_text(text)
        subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                        str(src), "-o", str(lib)], check=True, capture_output=True)
    h = C.CDLL(str(lib))
    h.symgb_host_group.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint]
    return h


def padded_tables(w):
    """Index and constant tables with every kernel row padded to a multiple of 4
    entries, the last entry repeated (the grouped layout's copies)."""
    d = w.plan.contents
    p, c = np.asarray(w.index_data, np.uint32), np.asarray(w.const_data, np.float64)
    p4, c4 = [], []
    for k in range(d.num_kernels):
        kd = d.kernels[k]
        n = int(kd.num_instances)
        stride = (n + 3) // 4 * 4
        for tab, out, off, rows in ((p, p4, kd.index_offset, kd.num_index_rows),
                                    (c, c4, kd.constants_offset, kd.num_constant_rows)):
            for r in range(rows):
                row = tab[off + r * n: off + (r + 1) * n]
                out.append(np.concatenate([row, np.repeat(row[-1:], stride - n)]) if n else row)
    cat = lambda parts, dt: np.concatenate(parts).astype(dt) if parts else np.zeros(1, dt)
    return cat(p4, np.uint32), cat(c4, np.float64)


def run_generated_grouped(w, inputs, math, S=1, items=4):
    """run_generated with the grouped item layout's bodies and padded tables."""
    u = native.Unit.from_workload(w, init=False)
    u.set_schedule(kind=native.SCHEDULE_PLAIN, math=math, items_per_thread=items)
    u.set_num_sets(S)
    u.set_item_layout(native.ITEMS_GROUPED)
    src = u.compiled_source(native.SCHEDULE_PLAIN)
    d = w.plan.contents
    lib = grouped_host_library(src, d.num_kernels, items)
    x = np.zeros(int(d.num_total_memory) * S)
    for i, a in enumerate(inputs):
        start = int(d.arg_start[i])
        per_set = np.asarray(a).reshape(S, -1)
        for s in range(S):
            x[(start + np.arange(per_set.shape[1])) * S + s] = per_set[s]
    p4, c4 = padded_tables(w)
    for k in range(d.num_kernels):
        n = int(d.kernels[k].num_instances)
        lib.symgb_host_group(k, x.ctypes.data, x.ctypes.data, p4.ctypes.data, c4.ctypes.data, (n + items - 1) // items, S)
    ids = np.asarray(w.out_index_data[int(d.output_start[0]):int(d.output_start[0]) + int(d.output_length[0])],
                     np.int64)
    return np.stack([x[ids * S + s] for s in range(S)])


def split_inputs(w, flat):
    out, off = [], 0
    for a in w.inputs:
        out.append(flat[off:off + len(a)])
        off += len(a)
    return out


def rel_err(a, ref, floor_frac=1e-10):
    floor = floor_frac * np.max(np.abs(ref))
    return float(np.max(np.abs(a - ref) / np.maximum(np.abs(ref), floor)))


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_generated_exact_bodies_reproduce_golden_results(name, size, seed):
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    out = run_generated(w, split_inputs(w, inp), native.MATH_EXACT)[0]
    assert np.array_equal(out.view(np.uint64), gold.view(np.uint64))


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
def test_generated_fast_bodies_within_tolerance(name, size, seed):
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    out = run_generated(w, split_inputs(w, inp), native.MATH_FAST)[0]
    assert rel_err(out, gold, FAST_FLOOR.get(name, 1e-10)) <= 1e-12


@pytest.mark.parametrize("name,size", [("cotan", 30), ("cloth", 9), ("ata", 30), ("neohookean", 3),
                                       ("random", 2000), ("literals", 300)])
def test_generated_exact_bodies_match_oracle(name, size):
    w = native.Workload(name, size, 9)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    out = run_generated(w, w.inputs, native.MATH_EXACT)[0]
    assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))


def test_generated_value_sets_are_independent():
    """Three value sets in one module: each set equals its own one-set evaluation."""
    w = native.Workload("cotan", 8, 22)
    rng = np.random.default_rng(5)
    sets = [w.inputs[0] * (1 + 0.01 * s) + rng.uniform(-1e-3, 1e-3, len(w.inputs[0])) for s in range(3)]
    out = run_generated(w, [np.concatenate(sets)], native.MATH_EXACT, S=3)
    for s in range(3):
        one = run_generated(w, [sets[s]], native.MATH_EXACT)[0]
        assert np.array_equal(out[s].view(np.uint64), one.view(np.uint64))


@pytest.mark.parametrize("name,size,seed", [("cotan", 8, 22), ("cloth", 5, 32), ("neohookean", 1, 41)])
@pytest.mark.parametrize("math", [0, 1])
def test_nvrtc_compiles_every_schedule(name, size, seed, math):
    w = native.Workload(name, size, seed)
    u = native.Unit.from_workload(w, init=False)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=math, items_per_thread=1 if math == 0 else 4)
    u.set_num_sets(1 if math == 0 else 5)
    for kind in (native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT):
        assert u.compile_check(kind) >= 0.0


def test_generated_source_folds_plan_constants():
    """Table offsets, instance counts and output slots are literals of the
    source, each index row is read once, and the entry points are the plan's
    kernels (plain) or levels."""
    w = native.Workload("cotan", 8, 22)
    u = native.Unit.from_workload(w, init=False)
    src = u.compiled_source(native.SCHEDULE_PLAIN)
    d = w.plan.contents
    assert len(re.findall(r'extern "C" __global__', src)) == sum(
        1 for k in range(d.num_kernels) if d.kernels[k].num_instances)
    for k in range(d.num_kernels):
        body = src[src.index(f"// kernel {k}:"):]
        body = body[:body.index("}\n")]
        rows = re.findall(r"__ldg\(p \+ (\d+)ull \+ i\)", body)
        assert len(rows) == len(set(rows))
    lv = u.compiled_source(native.SCHEDULE_LEVELS)
    assert len(re.findall(r'extern "C" __global__', lv)) == len({d.kernels[k].level for k in range(d.num_kernels)})


def test_items_per_thread_cover_every_work_item():
    """With several items per thread, each kernel's launch still covers its
    n x S work items: the module compiles and its block counts match."""
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w, init=False)
    for items in (1, 2, 4):
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_EXACT, items_per_thread=items,
                       threads_per_block=96)
        u.set_num_sets(3)
        src = u.compiled_source(native.SCHEDULE_PLAIN)
        assert f"* {96 * items}ull + threadIdx.x" in src
        if items > 1:
            assert f"for (int j = 0; j < {items}; ++j)" in src


def test_minimum_blocks_per_sm_become_launch_bounds():
    """blocks_per_sm > 0 compiles every entry point for that many resident
    CTAs per SM (capped at the SM's 2048 threads); the module still compiles."""
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w, init=False)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, threads_per_block=128, blocks_per_sm=6)
    src = u.compiled_source(native.SCHEDULE_PLAIN)
    assert "__launch_bounds__(128, 6)" in src and "__launch_bounds__(128)" not in src
    assert u.compile_check(native.SCHEDULE_PLAIN) >= 0.0
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, threads_per_block=512, blocks_per_sm=6)
    assert "__launch_bounds__(512, 4)" in u.compiled_source(native.SCHEDULE_LEVELS)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, threads_per_block=128)
    assert "__launch_bounds__(128)" in u.compiled_source(native.SCHEDULE_PLAIN)


def test_light_templates_get_an_unguarded_items_loop():
    """With several items per thread, a light template's threads whose items
    are all in range run them without per-item bounds checks (so their loads
    can be issued together); heavy templates keep the guarded loop only."""
    w = native.Workload("cloth", 5, 32)
    u = native.Unit.from_workload(w, init=False)
    u.set_schedule(kind=native.SCHEDULE_PLAIN, math=native.MATH_FAST, threads_per_block=64, items_per_thread=4)
    u.set_num_sets(8)
    src = u.compiled_source(native.SCHEDULE_PLAIN)
    kernels = {m.group(1): src[m.start():src.index("\n}\n", m.start())]
               for m in re.finditer(r'void __launch_bounds__\(64\) (symgb_k\d+)', src)}
    light = [k for k, body in kernels.items() if "} else {" in body]
    heavy = [k for k, body in kernels.items() if "} else {" not in body]
    assert light and heavy
    for k in light:
        body = kernels[k]
        assert "if (w0 + 192ull < " in body
    assert u.compile_check(native.SCHEDULE_PLAIN) >= 0.0
    assert u.compile_check(native.SCHEDULE_PERSISTENT) >= 0.0


@pytest.mark.parametrize("path,intrinsic", [(0, "__ldg"), (1, "__ldca"), (2, "__ldcg")])
def test_load_path_selects_the_load_intrinsic(path, intrinsic):
    """symgb_set_load_path picks the data path of every table and gather load
    of the generated module; each variant compiles for sm_103a."""
    w = native.Workload("cotan", 8, 22)
    u = native.Unit.from_workload(w, init=False)
    u.set_load_path(path)
    src = u.compiled_source(native.SCHEDULE_LEVELS)
    assert f"#define SYMGB_LD(a) {intrinsic}(a)" in src
    assert u.compile_check(native.SCHEDULE_LEVELS) >= 0.0
    assert native.symgb().symgb_set_load_path(u.handle, 3) == -1


@pytest.mark.parametrize("name,size,seed", GOLDEN_CASES)
@pytest.mark.parametrize("items", [1, 2, 4])
def test_grouped_bodies_reproduce_golden_results(name, size, seed, items):
    """The grouped item layout (a thread evaluates consecutive instances, its
    table entries read from padded rows) gives the reference's results bit
    for bit, including the last, partial group of every kernel."""
    _, inp, gold = load_golden(name, size)
    w = native.Workload(name, size, seed)
    out = run_generated_grouped(w, split_inputs(w, inp), native.MATH_EXACT, items=items)[0]
    assert np.array_equal(out.view(np.uint64), gold.view(np.uint64))


def test_grouped_bodies_with_value_sets_match_oracle():
    w = native.Workload("cloth", 9, 5)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    out = run_generated_grouped(w, [np.tile(a, 3) for a in w.inputs], native.MATH_EXACT, S=3, items=4)
    for s in range(3):
        assert np.array_equal(out[s].view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("kind", [native.SCHEDULE_PLAIN, native.SCHEDULE_LEVELS, native.SCHEDULE_PERSISTENT])
def test_grouped_modules_compile(kind):
    """Grouped modules compile for sm_103a in every schedule (vector loads of
    1, 2 and 4 entries)."""
    w = native.Workload("neohookean", 1, 41)
    u = native.Unit.from_workload(w, init=False)
    u.set_item_layout(native.ITEMS_GROUPED)
    for items in (1, 2, 4):
        u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST, items_per_thread=items)
        u.set_num_sets(1 if items < 4 else 64)
        src = u.compiled_source(kind)
        assert "symgbLoadIdx<IT>" in src and f", {items}, " in src
        assert u.compile_check(kind) >= 0.0
    assert native.symgb().symgb_set_item_layout(u.handle, 2) == -1


def test_generated_bodies_at_ata_stated_size():
    """B = A^T A + A at its stated size (A 10,000 x 10,000, 69,600 nonzeros;
    B 365,700): the generated bodies in exact mode reproduce the oracle bit
    for bit; in fast mode (here bit-identical to the device: only adds,
    multiplies and FMAs) within 1e-12 relative at the assembled matrices'
    floor of 1e-4 of the largest entry."""
    w = native.Workload("ata", 100, 2024)
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    exact = run_generated(w, w.inputs, native.MATH_EXACT)[0]
    assert np.array_equal(exact.view(np.uint64), ref.view(np.uint64))
    fast = run_generated(w, w.inputs, native.MATH_FAST)[0]
    assert rel_err(fast, ref, 1e-4) <= 1e-12
