#!/usr/bin/env bash
# Oracle test infrastructure: builds the UNMODIFIED reference sources (read in place
# under the reference checkout) together with oracle/ref_driver.cpp and the MKL /
# SuiteSparse / tictoc stand-ins in oracle/shim into oracle/_ref/libref.so.
# Nothing is copied out of the reference tree; outputs go to oracle/_ref/ only.
#
#   oracle/build_ref.sh [REFERENCE_DIR]        (default /root/reference)
#
# Flags follow the reference's Release build (CMakeLists.txt:19): -O3 -funroll-loops
# -march=native -ffast-math, plus -fopenmp (src/CMakeLists.txt:12).  A second library,
# libref_strict.so, is built with -O2 -ffp-contract=off (no fast-math, no FMA) for
# rounding analysis.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/ilu_solver.cpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 1
fi
mkdir -p "$OUT"
SRCS=("$REF/src/csr_matrix.cpp" "$REF/src/iluk.cpp" "$REF/src/ilu_solver.cpp" "$REF/src/gmres.cpp"
      "$REF/src_c/ilu_solver_c.cpp" "$REF/src_c/gmres_c.cpp" "$HERE/ref_driver.cpp")
INC=(-I"$HERE/shim" -I"$REF/include" -I"$REF/include_c" -I"$REF/src")
COMMON=(-std=c++17 -fPIC -shared -fopenmp -include cstdio -include cstdlib -w)
g++ "${COMMON[@]}" -O3 -funroll-loops -march=native -ffast-math -DNDEBUG "${INC[@]}" "${SRCS[@]}" \
    -o "$OUT/libref.so.tmp" -Wl,--no-undefined -lgomp -lm
mv "$OUT/libref.so.tmp" "$OUT/libref.so"
g++ "${COMMON[@]}" -O2 -ffp-contract=off -DNDEBUG "${INC[@]}" "${SRCS[@]}" \
    -o "$OUT/libref_strict.so.tmp" -Wl,--no-undefined -lgomp -lm
mv "$OUT/libref_strict.so.tmp" "$OUT/libref_strict.so"
echo "built $OUT/libref.so $OUT/libref_strict.so"
