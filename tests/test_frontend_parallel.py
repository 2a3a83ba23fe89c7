"""The front end's parallel passes (the cloth model's per-face blocks,
makeFixed numbering and column assembly; lockstep walk over kernel
instances; block extraction; release of the expression graph) give the same
plan as running them on one thread."""
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import hashlib, sys
sys.path.insert(0, sys.argv[1])
from symboliclib_gb300 import native
for c in [("cloth", 14, 7), ("cotan", 40, 5), ("neohookean", 3, 9), ("random", 20000, 22), ("random", 20000, 28)]:
    w = native.Workload(*c, text=True)
    print(c, hashlib.sha1(w.plan_text.encode()).hexdigest())
"""


def plan_hashes(threads: int) -> str:
    env = dict(os.environ, SYMGB_THREADS=str(threads))
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout


def test_parallel_front_end_matches_serial():
    serial = plan_hashes(1)
    assert serial.count("\n") == 5
    assert plan_hashes(4) == serial
    assert plan_hashes(13) == serial


CONCURRENT = r"""
import hashlib, sys
from concurrent.futures import ThreadPoolExecutor
sys.path.insert(0, sys.argv[1])
from symboliclib_gb300 import native
cases = [("cloth", 14, 7), ("cotan", 40, 5), ("neohookean", 3, 9), ("cloth", 9, 2), ("ata", 20, 4), ("cotan", 21, 8)]
def plan(c):
    return hashlib.sha1(native.Workload(*c, text=True).plan_text.encode()).hexdigest()
serial = [plan(c) for c in cases]
with ThreadPoolExecutor(max_workers=4) as ex:
    for rep in range(2):
        assert list(ex.map(plan, cases)) == serial, rep
print("ok")
"""


def test_front_ends_side_by_side_match_serial():
    """Several front ends building at once on different threads (their
    makeFixed numbering is per thread) give each workload the plan it gets
    when built alone."""
    env = dict(os.environ, SYMGB_THREADS="4")
    r = subprocess.run([sys.executable, "-c", CONCURRENT, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("ok")
