#!/bin/sh
# Builds the reference's own execution paths for one workload from the source
# its ComputeUnit generated (oracle/ref_codegen.cpp keeps it in <gen_dir>), and
# the timing driver oracle/ref_run.cpp.  Runs next to the GPU (aarch64 too): no
# file of the reference is needed there, only <gen_dir>.
#
#   oracle/ref_paths.sh <gen_dir> cuda     # cudaCode.cu ->
#       ref_default.so : the reference's nvcc command (ComputeUnit.cpp:121):
#                        nvcc -O3 -Xcompiler '-fPIC -shared', no -arch
#                        (compute_75 PTX, JIT-compiled by the driver)
#       ref_sm103a.so  : the same with -arch=sm_103a
#       ref_exact.so   : -arch=sm_103a --fmad=false (every operation rounded as
#                        written: the bit-exact reference)
#   oracle/ref_paths.sh <gen_dir> cpu      # cpuCode.cpp ->
#       ref_cpu.so     : the reference's clang++ command (ComputeUnit.cpp:125-132)
#                        mapped onto g++ by ref_clangxx.sh (x86 -m flags dropped
#                        on other machines, libgomp for libiomp5), with
#                        -DNUMTHREADS=<host cores> (NUMTHREADS env to override)
# plus <gen_dir>/ref_run (ref_run.cpp; -DREF_CUDA for cuda).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
GEN=$(cd "$1" && pwd)
KIND=$2
NVCC=${NVCC:-nvcc}
if [ "$KIND" = "cuda" ]; then
  cd "$GEN"
  $NVCC -I"$HERE/ref_shim" -Xcompiler '-fPIC -shared' -O3 -o ref_default.so cudaCode.cu &
  $NVCC -I"$HERE/ref_shim" -Xcompiler '-fPIC -shared' -O3 -arch=sm_103a -o ref_sm103a.so cudaCode.cu &
  $NVCC -I"$HERE/ref_shim" -Xcompiler '-fPIC -shared' -O3 -arch=sm_103a --fmad=false -o ref_exact.so cudaCode.cu &
  $NVCC -O2 -DREF_CUDA -o ref_run "$HERE/ref_run.cpp" -ldl &
  wait
  test -f ref_default.so && test -f ref_sm103a.so && test -f ref_exact.so && test -f ref_run
elif [ "$KIND" = "cpu" ]; then
  cd "$GEN"
  N=${NUMTHREADS:-$(nproc)}
  sh "$HERE/ref_clangxx.sh" -shared -fPIC -ffast-math -fno-trapping-math -fno-math-errno -fno-signed-zeros -O3 \
     -std=c++17 -msse4.2 -mavx2 -mfma cpuCode.cpp -oref_cpu.so -DNUMTHREADS=$N -fopenmp &
  g++ -O2 -o ref_run_cpu "$HERE/ref_run.cpp" -ldl &
  wait
  test -f ref_cpu.so && test -f ref_run_cpu
else
  echo "usage: ref_paths.sh <gen_dir> cuda|cpu" >&2
  exit 2
fi
