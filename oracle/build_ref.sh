#!/usr/bin/env bash
# Build the UNMODIFIED reference DistPCA sources as a CPU oracle (test
# infrastructure only).  Sources are compiled where they lie under the
# reference checkout; every output goes to oracle/_ref/ (git-ignored).
#
#   oracle/_ref/DistPCA.exe   the reference command line, single rank
#   oracle/_ref/ref_harness   golden-vector dumper (oracle/ref_harness.cpp)
#
# MPI is replaced by oracle/shim/mpi.h (one rank, pread for MPI-IO) and
# MKL/OpenBLAS by scipy's bundled OpenBLAS through oracle/shim/*.h.
# Flags follow the reference Makefile's Linux branch (-O3, no -fopenmp).
#
# The checkout is $DPCA_REFERENCE, else the one this recipe was written against.  Options:
#   --if-present   exit 0 without building when the checkout is absent (the GPU machine has none)
#   --print-ref    print the checkout directory and exit (scripts that read the reference's
#                  files, such as tests/golden/make_golden.py, ask this recipe for it)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${DPCA_REFERENCE:-/root/reference}"
OUT="$HERE/_ref"
SRC="$REF/src"
if [ "${1:-}" = "--print-ref" ]; then
    echo "$REF"
    exit 0
fi
if [ ! -f "$SRC/methods.cpp" ]; then
    if [ "${1:-}" = "--if-present" ]; then
        echo "build_ref.sh: no reference checkout at $REF; oracle/_ref not built"
        exit 0
    fi
    echo "build_ref.sh: reference sources not found under $REF" >&2
    exit 1
fi
BLAS="$(python3 "$HERE/find_openblas.py")"
BLASDIR="$(dirname "$BLAS")"
mkdir -p "$OUT/obj"
ARCH="$(uname -m)"
if [ "$ARCH" = "x86_64" ]; then
    CXXF="-O3 -std=c++11 -mavx2 -mfma -march=native"
else
    CXXF="-O3 -std=c++11"
fi
INC="-I$HERE/shim -I$SRC"
pids=()
for f in distpca utilities methods; do
    g++ $CXXF $INC -c "$SRC/$f.cpp" -o "$OUT/obj/$f.o" & pids+=($!)
done
for f in gaussian gennorm io; do
    gcc -O3 -fPIE $INC -c "$SRC/$f.c" -o "$OUT/obj/$f.o" & pids+=($!)
done
gcc -O2 -c "$HERE/shim/openblas_compat.c" -o "$OUT/obj/openblas_compat.o" & pids+=($!)
g++ $CXXF $INC -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
LIBS="$BLAS -Wl,-rpath,$BLASDIR -lgomp -lpthread -lm"
O="$OUT/obj"
g++ -o "$OUT/DistPCA.exe" $O/distpca.o $O/utilities.o $O/methods.o $O/gaussian.o $O/gennorm.o $O/io.o \
    $O/openblas_compat.o $LIBS
g++ -o "$OUT/ref_harness" $O/ref_harness.o $O/utilities.o $O/gennorm.o $O/openblas_compat.o $LIBS
echo "built $OUT/DistPCA.exe and $OUT/ref_harness"
