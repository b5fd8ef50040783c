#!/bin/sh
# Builds the CPU oracle (test infrastructure: the checker of the GPU
# solver and the bench's CPU baseline) into oracle/_build/liboracle.so.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O3 -fopenmp -fPIC -shared -Wall "$HERE/oracle.cpp" -o "$HERE/_build/liboracle.so"
echo "$HERE/_build/liboracle.so"
