"""The C++ API (include/symgb/ComputeUnit.hpp, differentiation.hpp) compiled
into a program: the reference Tutorial's known answers on the CPU, and a
ComputeUnit compile/execute/getResults round trip on the GPU; the front end's
parallel CRC-64 vector hash against the serial one."""
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT
from symboliclib_gb300 import build

SRC = ROOT / "tests" / "cpp" / "tutorial.cpp"


@pytest.fixture(scope="module")
def tutorial_binary():
    out = build.OBJ / "tutorial_test"
    lib = build.LIB
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", f"-I{ROOT / 'include'}", str(SRC), "-o", str(out),
           f"-L{lib}", "-lsymgb", f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_tutorial_known_answers(tutorial_binary):
    r = subprocess.run([str(tutorial_binary)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_exit_error_policy_exits_like_the_reference(tutorial_binary):
    """OnError(ErrorPolicy::Exit): an engine error prints the message and ends
    the process with a failure status, as the reference's generated library
    does; the default policy throws and Print carries on (checked inside)."""
    r = subprocess.run([str(tutorial_binary), "--exit-policy"], capture_output=True, text=True)
    assert r.returncode == 1, r.stdout + r.stderr
    assert "symgb:" in r.stderr and "not reached" not in r.stdout


@pytest.mark.gpu
def test_compute_unit_round_trip(tutorial_binary):
    r = subprocess.run([str(tutorial_binary), "--gpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_parallel_vector_hash_equals_serial():
    out = build.OBJ / "crc_combine_test"
    lib = build.LIB
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "crc_combine.cpp"), "-o",
           str(out), f"-L{lib}", "-lsymgb", f"-Wl,-rpath,{lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
