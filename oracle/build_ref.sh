#!/bin/sh
# Builds oracle/_ref/libsonar_ref.so from the reference's own sources where they
# lie (test infrastructure: it pins the oracle and writes tests/golden/).
# Usage: oracle/build_ref.sh REFERENCE_ROOT  (or SONAR_REFERENCE_ROOT in the
# environment); without either it builds nothing.
# The reference's unmodified src/Facet.cpp, src/Globals.cpp and src/OptiX.cu are
# compiled as host C++ with oracle/ref_harness.cpp; oracle/ref_shim/ stands in
# for the OptiX and GL headers.  No fused multiply-add, like the reference's
# x86-64 host build.  Exits 0 without building when the sources are absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${SONAR_REFERENCE_ROOT:-}}
if [ -z "$REF" ]; then
    echo "build_ref: no reference root given; skipped"
    exit 0
fi
SRC="$REF/src"
if [ ! -f "$SRC/Facet.cpp" ] || [ ! -f "$SRC/OptiX.cu" ]; then
    echo "build_ref: reference sources not found under $REF; skipped"
    exit 0
fi
CUDA=${CUDA_HOME:-/usr/local/cuda}
OUT="$HERE/_ref"
mkdir -p "$OUT"
FLAGS="-O2 -std=c++17 -fPIC -ffp-contract=off -w -include cuda_runtime.h -I$HERE/ref_shim -I$SRC -I$CUDA/include -I$CUDA/include/cccl"
g++ $FLAGS -c "$SRC/Facet.cpp" -o "$OUT/Facet.o"
g++ $FLAGS -c "$SRC/Globals.cpp" -o "$OUT/Globals.o"
g++ $FLAGS -x c++ -c "$SRC/OptiX.cu" -o "$OUT/OptiX.o"
g++ $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o"
g++ -shared -o "$OUT/libsonar_ref.so" "$OUT/Facet.o" "$OUT/Globals.o" "$OUT/OptiX.o" "$OUT/ref_harness.o"
rm -f "$OUT"/*.o
echo "build_ref: $OUT/libsonar_ref.so"
