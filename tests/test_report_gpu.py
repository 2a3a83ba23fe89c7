"""The measurement reports of symboliclib_gb300.report on small cases: the
uneven multi-pattern batch with autotuned schedules, replayed as one CUDA
graph, agrees with the FP64 numeric model."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT


@pytest.mark.gpu
def test_tuned_batch_report():
    r = subprocess.run([sys.executable, "-m", "symboliclib_gb300.report", "batch", "--count", "6", "--min-side", "4",
                        "--max-side", "9", "--max-sets", "3", "--steps", "2"], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["instances"] == 6
    assert sum(line["graph"]["schedule"].values()) == line["distinct_patterns"]
    assert line["max_rel_err_sampled"] <= 1e-12
    assert line["graph"]["ms"] > 0
