#!/bin/sh
# Keeps the reference's generated code and table files for the benchmark
# workloads in oracle/_ref/gen/<workload>_<size>_<cuda|cpu>/ (see
# oracle/ref_paths.py).  Needs the reference sources (REF, default
# /root/reference) to build oracle/_ref/libsymref.so; run where they are
# mounted, before the directories are taken to the machine with the GPU.
#
#   oracle/ref_generate.sh [workload:size:seed ...]
#   (default: cotan:500:2024 cloth:300:2024, both devices)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${REF:-/root/reference}
make -s -C "$HERE" codegen REF="$REF"
SPECS=${*:-"cotan:500:2024 cloth:300:2024"}
for spec in $SPECS; do
  w=$(echo "$spec" | cut -d: -f1)
  n=$(echo "$spec" | cut -d: -f2)
  seed=$(echo "$spec" | cut -d: -f3)
  for dev in cuda cpu; do
    d="$HERE/_ref/gen/${w}_${n}_${dev}"
    mkdir -p "$d"
    if [ "$dev" = "cuda" ]; then param=128; else param=4; fi
    "$HERE/_ref/ref_codegen" "$d" "$w" "$n" "$seed" "$dev" "$param"
  done
done
