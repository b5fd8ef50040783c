#!/bin/sh
# Builds the reference's own code, compiled in place from the reference
# checkout (PPS_REFERENCE; default: a `reference` directory beside this
# repository), into oracle/_ref/ (git-ignored). TEST INFRASTRUCTURE ONLY: these programs
# generate and pin the golden fixtures under tests/golden/; no product code
# links or runs them.
#
#   oracle/_ref/ref_capture  reference tree compiler on a host CUDA stub
#   oracle/_ref/tiny_check   reference known-answer EV program
#   oracle/_ref/ref_probe    reference evaluator / betActions / range parser
#   oracle/_ref/gpu_cfr_kernels.fatbin
#                            the reference's GPU kernels (cuda/gpu_cfr.cu,
#                            device code only) for sm_103a, run on the GPU by
#                            oracle/ref/ref_gpu.cpp as a second checker and
#                            timed beside the CPU port
#
# Only the reference checkout's own files are compiled; its build system
# (CMake/Makefile) is not used.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${PPS_REFERENCE:-$HERE/../../../reference}"
OUT="$HERE/../_ref"
if [ ! -d "$REF/cuda" ]; then
  echo "reference sources not found at $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
CORE="$REF/src/postflop_cfr.cpp $REF/src/cards.cpp $REF/src/range.cpp $REF/src/common.cpp"
nvcc -std=c++17 -O1 -w -gencode arch=compute_103a,code=sm_103a -cudart none \
  -I"$REF/src" -I"$REF/cuda" \
  "$HERE/ref_capture.cu" "$HERE/cuda_host_stub.cpp" $CORE \
  -o "$OUT/ref_capture"
g++ -std=c++17 -O2 -w -I"$REF/src" "$REF/tools/tiny_check.cpp" \
  "$REF/src/cards.cpp" "$REF/src/range.cpp" "$REF/src/common.cpp" \
  -o "$OUT/tiny_check"
g++ -std=c++17 -O2 -w -I"$REF/src" "$HERE/ref_probe.cpp" $CORE \
  -o "$OUT/ref_probe"
nvcc -std=c++17 -O3 -w -fatbin -gencode arch=compute_103a,code=sm_103a \
  -I"$REF/src" -I"$REF/cuda" "$REF/cuda/gpu_cfr.cu" -o "$OUT/gpu_cfr_kernels.fatbin"
"$OUT/ref_capture" --treebuf > "$OUT/treebuf.txt"
echo "built $OUT/ref_capture $OUT/tiny_check $OUT/ref_probe $OUT/gpu_cfr_kernels.fatbin"
