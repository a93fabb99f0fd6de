#!/bin/sh
# Builds the reference's own FP64 CPU calculation path (test oracle only) into
# oracle/_ref/libscref.so, straight from the reference sources where they lie.
# The reference tree is read-only and is not copied: g++ reads the two
# translation units below in place. The .cu file is compiled as plain C++,
# which leaves exactly the reference's CPU path (no __CUDACC__).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -e
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/Source/sc_calc_generic_cpu.cpp" ]; then
    echo "reference sources not found under $REF; oracle/_ref not built" >&2
    exit 3
fi
mkdir -p "$OUT"
CXXFLAGS="-O2 -std=gnu++17 -fPIC -ffp-contract=off -w -I$HERE/ref_stubs -I$REF/Source"
g++ $CXXFLAGS -c -x c++ "$REF/Source/sc_calc_generic_cpu.cpp" -o "$OUT/sc_calc_generic_cpu.o" &
g++ $CXXFLAGS -c -x c++ "$REF/Source/sc_calc_generic_gpu.cu" -o "$OUT/sc_calc_generic_gpu.o" &
g++ $CXXFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" &
wait
g++ -shared -o "$OUT/libscref.so" "$OUT/sc_calc_generic_cpu.o" "$OUT/sc_calc_generic_gpu.o" "$OUT/ref_driver.o" -lpthread
echo "built $OUT/libscref.so"
