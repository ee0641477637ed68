#!/usr/bin/env bash
# Oracle test infrastructure: builds the CPU restatement oracle/port/ilu_port.cpp into
# oracle/_build/libport.so (host compiler only; runs on x86_64 and aarch64 alike).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
g++ -std=c++17 -O3 -fPIC -shared -fopenmp "$HERE/port/ilu_port.cpp" -o "$HERE/_build/libport.so.tmp" -Wl,--no-undefined
mv "$HERE/_build/libport.so.tmp" "$HERE/_build/libport.so"
echo "built $HERE/_build/libport.so"
