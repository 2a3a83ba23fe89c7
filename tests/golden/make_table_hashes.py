"""Records SHA-256 digests of the reference's own table files (indexData,
outIndexData, constData: the tables its ComputeUnit writes, Utilities.hpp:156-161)
for the benchmark workloads into tests/golden/reference_tables.json.

Run after oracle/ref_generate.sh, which keeps those files (produced by the
reference library built from its sources) in oracle/_ref/gen/.  The tests
compare the engine front end's tables at the same sizes against these
digests, so the front end is pinned to the reference at full size without
the reference being present."""
import hashlib
import json
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
GEN = ROOT / "oracle" / "_ref" / "gen"
OUT = Path(__file__).resolve().parent / "reference_tables.json"


def main():
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    for d in sorted(GEN.iterdir()):
        if not (d / "indexData").exists():
            continue
        entry = {}
        for name in ("indexData", "outIndexData", "constData", "inputs.bin"):
            b = (d / name).read_bytes()
            entry[name] = {"bytes": len(b), "sha256": hashlib.sha256(b).hexdigest()}
        data[d.name] = entry
    OUT.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
    print(f"{len(data)} workloads -> {OUT}")


if __name__ == "__main__":
    main()
