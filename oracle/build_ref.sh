#!/bin/sh
# Builds the reference's own FP64 CPU calculation path (test oracle only) into
# oracle/_ref/libscref.so (its r-phi transform into libscpost.so, its
# downhill simplex into libscsimplex.so),
# straight from the reference sources where they lie.
# The reference tree is read-only and is not copied: g++ reads the two
# translation units below in place. The .cu file is compiled as plain C++,
# which leaves exactly the reference's CPU path (no __CUDACC__).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The reference root is the argument, else $CS_REFERENCE_ROOT, else
# /root/reference. Exit status 3: no reference sources there (nothing built).
set -e
REF="${1:-${CS_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/Source/sc_calc_generic_cpu.cpp" ]; then
    echo "reference sources not found under $REF; oracle/_ref not built" >&2
    exit 3
fi
mkdir -p "$OUT"
# Q_OS_LINUX: the platform macro a Linux Qt build defines (it selects the "\n"
# line end of the reference's log texts)
CXXFLAGS="-O2 -std=gnu++17 -fPIC -ffp-contract=off -w -DQ_OS_LINUX -I$HERE/ref_stubs -I$REF/Source"
g++ $CXXFLAGS -c -x c++ "$REF/Source/sc_calc_generic_cpu.cpp" -o "$OUT/sc_calc_generic_cpu.o" &
g++ $CXXFLAGS -c -x c++ "$REF/Source/sc_calc_generic_gpu.cu" -o "$OUT/sc_calc_generic_gpu.o" &
g++ $CXXFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" &
wait
g++ -shared -o "$OUT/libscref.so" "$OUT/sc_calc_generic_cpu.o" "$OUT/sc_calc_generic_gpu.o" "$OUT/ref_driver.o" -lpthread
echo "built $OUT/libscref.so"
# probe build: the same sources without builtins (every math call stays a
# call), linked with one-ulp wrappers of the math library (ref_probe.c)
PFLAGS="$CXXFLAGS -fno-builtin"
g++ $PFLAGS -c -x c++ "$REF/Source/sc_calc_generic_cpu.cpp" -o "$OUT/probe_cpu.o" &
g++ $PFLAGS -c -x c++ "$REF/Source/sc_calc_generic_gpu.cu" -o "$OUT/probe_gpu.o" &
g++ $PFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/probe_driver.o" &
gcc -O2 -fPIC -c "$HERE/ref_probe.c" -o "$OUT/ref_probe.o" &
wait
WRAP="-Wl,--wrap=sin,--wrap=cos,--wrap=atan,--wrap=atan2,--wrap=pow,--wrap=exp,--wrap=log,--wrap=acos"
g++ -shared $WRAP -o "$OUT/libscref_probe.so" "$OUT/probe_cpu.o" "$OUT/probe_gpu.o" "$OUT/probe_driver.o" \
    "$OUT/ref_probe.o" -lpthread -lm
echo "built $OUT/libscref_probe.so"
# the r-phi transform of the post-processing unit (its FFT needs FFTW, which
# is absent: fftw3.h in ref_stubs only lets the unit compile)
g++ $CXXFLAGS -c -x c++ "$REF/Source/sc_postproc.cpp" -o "$OUT/sc_postproc.o" &
g++ $CXXFLAGS -c "$HERE/ref_postproc.cpp" -o "$OUT/ref_postproc.o" &
wait
g++ -shared -o "$OUT/libscpost.so" "$OUT/sc_postproc.o" "$OUT/ref_postproc.o"
echo "built $OUT/libscpost.so"
# the downhill simplex (Source/sc_simplexfit2d.cpp) with the stand-in
# calculation class of ref_stubs/simplex_calc.h, forced in ahead of the unit
SFLAGS="$CXXFLAGS -DCONSOLENPROG"
g++ $SFLAGS -include "$HERE/ref_stubs/simplex_calc.h" -c -x c++ "$REF/Source/sc_simplexfit2d.cpp" \
    -o "$OUT/sc_simplexfit2d.o" &
g++ $SFLAGS -c "$HERE/ref_simplex.cpp" -o "$OUT/ref_simplex.o" &
wait
g++ -shared -o "$OUT/libscsimplex.so" "$OUT/sc_simplexfit2d.o" "$OUT/ref_simplex.o"
echo "built $OUT/libscsimplex.so"
# the measured-data file readers (Source/sc_readdata.cpp) with the Qt
# stand-ins of ref_stubs_io (HDF5 left out; the TIFF and 2D-SANS readers
# compile but are not run) and the console widImage stand-in forced in
RFLAGS="-O2 -std=gnu++17 -fPIC -w -DQ_OS_LINUX -I$HERE/ref_stubs_io -I$REF/Source -include $HERE/ref_stubs_io/readers_env.h"
g++ $RFLAGS -c -x c++ "$REF/Source/sc_readdata.cpp" -o "$OUT/sc_readdata.o" &
g++ $RFLAGS -c "$HERE/ref_readers.cpp" -o "$OUT/ref_readers.o" &
wait
g++ -shared -o "$OUT/libscreaders.so" "$OUT/sc_readdata.o" "$OUT/ref_readers.o"
echo "built $OUT/libscreaders.so"
