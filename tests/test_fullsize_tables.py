"""The front end at benchmark size, on the CPU: the index, output-index and
constant tables (and the seeded inputs) the engine's front end builds for
cotan 500x500, for B = A^T A + A at its stated size (A 10,000 x 10,000) and
for the Neo-Hookean Hessian of a 10 x 10 x 10 cube (5,000 tets) have the
SHA-256 digests of the tables the reference's own ComputeUnit wrote
for the same workloads, in its CUDA layout and in its CPU
ComputeUnit's VecWidth(4) layout (padded, blocked tables).  The digests are
recorded in tests/golden/reference_tables.json by
tests/golden/make_table_hashes.py from the reference's files.  The cloth
200x200 digests are checked with the GPU tests (test_fullsize_gpu.py), whose
host builds that front end in a fraction of the time."""
import hashlib
import json

import numpy as np
import pytest

from conftest import ROOT
from symboliclib_gb300 import native

TABLES = ROOT / "tests" / "golden" / "reference_tables.json"


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name,size", [("cotan", 500), ("ata", 100), ("neohookean", 10)])
@pytest.mark.parametrize("layout,width", [("cuda", 0), ("cpu", 4)])
def test_tables_equal_reference(name, size, layout, width):
    w = native.Workload(name, size, 2024, vector_width=width)
    ref = json.loads(TABLES.read_text())[f"{name}_{size}_{layout}"]
    assert digest(w.index_data) == ref["indexData"]["sha256"]
    assert digest(w.out_index_data) == ref["outIndexData"]["sha256"]
    assert digest(w.const_data) == ref["constData"]["sha256"]
    assert digest(np.concatenate(w.inputs)) == ref["inputs.bin"]["sha256"]


def test_ata100_oracle_against_numeric_model():
    """B = A^T A + A at its stated size: the oracle (the reference's strict
    operation order) against the FP64 numeric model (the role of Eigen's
    numeric A^T A + A in the reference's tutorial) within 1e-11 relative, with
    a floor of 1e-10 of the largest entry."""
    import oracle.cpu as ocpu
    w = native.Workload("ata", 100, 2024)
    assert len(w.numeric) == 365700 and sum(len(a) for a in w.inputs) == 69600
    ref = ocpu.evaluate(w.plan, w.index_data, w.out_index_data, w.const_data, w.inputs)[0]
    floor = 1e-10 * np.max(np.abs(w.numeric))
    assert np.max(np.abs(ref - w.numeric) / np.maximum(np.abs(w.numeric), floor)) <= 1e-11
