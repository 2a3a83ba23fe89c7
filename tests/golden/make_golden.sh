#!/bin/sh
# Regenerates the golden fixtures in tests/golden/ from the reference
# SymbolicLib.  Needs the reference sources (REF, default /root/reference);
# builds oracle/_ref/libsymref.so with oracle/Makefile, compiles gen_golden.cpp
# against it and runs it in a scratch directory (the reference writes its
# generated code and table files into the current directory).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
REF=${REF:-/root/reference}
make -s -C "$ROOT/oracle" ref REF="$REF"
OUTBIN="$ROOT/oracle/_ref/gen_golden"
(cd "$ROOT" && python3 -m symboliclib_gb300.build > /dev/null)
g++ -std=c++17 -O2 -w -I "$ROOT/oracle/eigen_stub" -I "$REF/src" "$HERE/gen_golden.cpp" \
    -L "$ROOT/oracle/_ref" -lsymref -Wl,-rpath,"$ROOT/oracle/_ref" \
    -L "$ROOT/symboliclib_gb300/lib" -lsymgb -Wl,-rpath,"$ROOT/symboliclib_gb300/lib" -o "$OUTBIN"
WORK=$(mktemp -d)
trap 'rm -rf "$WORK"' EXIT
cd "$WORK"
export PATH="$ROOT/oracle/_ref/bin:$PATH" SYMREF_STRICT=1
# workload size seed
for spec in "ata 6 11" "ata 9 12" "cotan 5 21" "cotan 8 22" "cloth 3 31" "cloth 5 32" "neohookean 1 41" \
            "neohookean 2 42" "cotan 40 23" "cloth 12 33" "neohookean 4 43"; do
  set -- $spec
  "$OUTBIN" "$HERE" "$1" "$2" "$3" > /dev/null
done
