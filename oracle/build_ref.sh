#!/usr/bin/env bash
# Oracle test infrastructure: builds the UNMODIFIED reference sources together with
# oracle/ref_driver.cpp and the MKL / SuiteSparse / tictoc stand-ins in oracle/shim.
# Outputs go to oracle/_ref/ only (git-ignored):
#
#   libref.so         reference flags (CMakeLists.txt:19: -O3 -funroll-loops
#                     -march=native -ffast-math, plus -fopenmp from src/CMakeLists.txt:12),
#                     serial BLAS-1 stand-ins (index-order sums); made the golden fixtures
#   libref_strict.so  -O2 -ffp-contract=off (no fast-math, no FMA), for rounding analysis
#   libref_omp.so     reference flags with OpenMP-threaded BLAS-1 stand-ins (MKL threads
#                     its BLAS-1 on long vectors); the CPU timing build
#
#   oracle/build_ref.sh [REFERENCE_DIR]
#
# REFERENCE_DIR defaults to $PAR_ILU0_REFERENCE_DIR, else /root/reference.  When the
# checkout is there, the sources are compiled where they lie and the files this build
# reads (and the reference's C test programs test/test.c, test/amd_test.c, which the
# tests compile unchanged against this library's headers) are also staged under
# oracle/_ref/src, so that a machine the working tree is
# copied to without the checkout can rebuild from the staged copy (the only other
# source this script accepts).  Nothing is copied into tracked files.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${PAR_ILU0_REFERENCE_DIR:-/root/reference}}"
OUT="$HERE/_ref"
STAGE="$OUT/src"
mkdir -p "$OUT"
if [ -f "$REF/src/ilu_solver.cpp" ]; then
    rm -rf "$STAGE.tmp"
    mkdir -p "$STAGE.tmp"
    cp -r "$REF/src" "$REF/include" "$REF/include_c" "$REF/src_c" "$STAGE.tmp/"
    mkdir -p "$STAGE.tmp/test"
    cp "$REF/test/test.c" "$REF/test/amd_test.c" "$STAGE.tmp/test/"
    rm -rf "$STAGE"
    mv "$STAGE.tmp" "$STAGE"
elif [ -f "$STAGE/src/ilu_solver.cpp" ]; then
    REF="$STAGE"
else
    echo "reference sources not found under $REF or $STAGE" >&2
    exit 1
fi
SRCS=("$REF/src/csr_matrix.cpp" "$REF/src/iluk.cpp" "$REF/src/ilu_solver.cpp" "$REF/src/gmres.cpp"
      "$REF/src_c/ilu_solver_c.cpp" "$REF/src_c/gmres_c.cpp" "$HERE/ref_driver.cpp")
INC=(-I"$HERE/shim" -I"$REF/include" -I"$REF/include_c" -I"$REF/src")
COMMON=(-std=c++17 -fPIC -shared -fopenmp -include cstdio -include cstdlib -w)
FAST=(-O3 -funroll-loops -march=native -ffast-math -DNDEBUG)
g++ "${COMMON[@]}" "${FAST[@]}" "${INC[@]}" "${SRCS[@]}" -o "$OUT/libref.so.tmp" -Wl,--no-undefined -lgomp -lm &
P1=$!
g++ "${COMMON[@]}" -O2 -ffp-contract=off -DNDEBUG "${INC[@]}" "${SRCS[@]}" \
    -o "$OUT/libref_strict.so.tmp" -Wl,--no-undefined -lgomp -lm &
P2=$!
g++ "${COMMON[@]}" "${FAST[@]}" -DSHIM_THREADED_BLAS "${INC[@]}" "${SRCS[@]}" \
    -o "$OUT/libref_omp.so.tmp" -Wl,--no-undefined -lgomp -lm &
P3=$!
wait $P1
wait $P2
wait $P3
mv "$OUT/libref.so.tmp" "$OUT/libref.so"
mv "$OUT/libref_strict.so.tmp" "$OUT/libref_strict.so"
mv "$OUT/libref_omp.so.tmp" "$OUT/libref_omp.so"
echo "built $OUT/libref.so $OUT/libref_strict.so $OUT/libref_omp.so (sources: $REF)"
