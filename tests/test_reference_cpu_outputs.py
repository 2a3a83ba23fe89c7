"""The oracle at larger sizes against the reference itself: the reference CPU
ComputeUnit's generated code for a workload (cpuCode.cpp and its tables, kept
by oracle/ref_generate.sh from the reference library built from its
sources), compiled by its own command line in strict mode (no fast-math, no
contraction: every operation rounded as written) and run through its five
library calls by oracle/ref_run.cpp, gives the oracle's results bit for bit.
Runs where that generated code is present (where the reference sources are
mounted); skipped elsewhere."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import ref_paths
from symboliclib_gb300 import native

import oracle.cpu as ocpu

CASES = [("ata", 100), ("neohookean", 10), ("cotan", 500)]


@pytest.mark.parametrize("name,size", CASES)
def test_reference_cpu_code_equals_oracle(name, size, tmp_path):
    if not ref_paths.available(name, size, "cpu"):
        pytest.skip("the reference's generated CPU code is not present here")
    gen = tmp_path / "gen"
    shutil.copytree(ref_paths.gen_dir(name, size, "cpu"), gen, ignore=shutil.ignore_patterns("*.so", "ref_run_cpu"))
    env = dict(os.environ, SYMREF_STRICT="1", NUMTHREADS="2")
    r = subprocess.run(["sh", str(ROOT / "oracle" / "ref_paths.sh"), str(gen), "cpu"], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    out = tmp_path / "results.bin"
    r = subprocess.run([str(gen / "ref_run_cpu"), str(gen), str(gen / "ref_cpu.so"), "0", "1", str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    ref = np.fromfile(out, np.float64)
    w = native.Workload(name, size, 2024)  # the oracle reads the device layout's tables
    assert np.array_equal(np.concatenate(w.inputs).view(np.uint64),
                          np.fromfile(gen / "inputs.bin", np.float64).view(np.uint64))
    oracle = np.concatenate(ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs))
    assert ref.shape == oracle.shape
    assert np.array_equal(ref.view(np.uint64), oracle.view(np.uint64))
