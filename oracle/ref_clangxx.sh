#!/bin/sh
# Stand-in for the `clang++` command line that the reference's
# ComputeUnit::compile builds (ComputeUnit.cpp:125-132).  Maps it onto g++:
#  - drops the /opt/rocm include/lib/rpath arguments and -liomp5 (uses libgomp);
#  - drops x86-only -m flags on other architectures;
#  - with SYMREF_STRICT=1: drops -ffast-math and adds -ffp-contract=off so every
#    floating-point operation is evaluated as written (IEEE, no FMA contraction).
args=""
arch=$(uname -m)
for a in "$@"; do
  case "$a" in
    -I/opt/rocm*|-L/opt/rocm*|-Wl,-rpath,/opt/rocm*|-liomp5) continue ;;
    -msse4.2|-mavx2|-mfma) [ "$arch" = "x86_64" ] || continue ;;
    -ffast-math|-fno-signed-zeros|-fno-trapping-math) [ "${SYMREF_STRICT:-0}" = "1" ] && continue ;;
  esac
  args="$args '$a'"
done
if [ "${SYMREF_STRICT:-0}" = "1" ]; then
  args="$args -ffp-contract=off"
fi
eval exec g++ $args -lgomp
