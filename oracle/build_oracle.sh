#!/bin/sh
# Builds the CPU oracle (test infrastructure: the reference against which
# the GPU solver is tested, and the bench's CPU baseline) into oracle/_build/liboracle.so, and
# the host runner of the reference's own GPU kernels (oracle/ref/ref_gpu.cpp,
# test and measurement infrastructure) into oracle/_build/libref_gpu.so.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O3 -fopenmp -fPIC -shared -Wall "$HERE/oracle.cpp" -o "$HERE/_build/liboracle.so"
if command -v nvcc > /dev/null 2>&1; then
  nvcc -std=c++17 -O2 -shared -Xcompiler -fPIC "$HERE/ref/ref_gpu.cpp" \
    -o "$HERE/_build/libref_gpu.so"
fi
echo "$HERE/_build/liboracle.so"
