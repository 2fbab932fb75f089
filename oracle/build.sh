#!/bin/sh
# Builds the CPU oracle (test infrastructure) twice:
#   oracle/_build/liboracle.so       parity: no -march=native and no fused
#                                    multiply-add, so that x86-64 and aarch64
#                                    hosts produce bit-identical results;
#   oracle/_build/liboracle_time.so  timing only (the CPU baseline): the
#                                    renderer's Release flags (src/CMakeLists.txt
#                                    -O3 -fno-strict-aliasing -fopenmp), the
#                                    compiler's default contraction (fused
#                                    multiply-add on AArch64), without
#                                    -march=native, which host code of this
#                                    project does not use.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CXX:-g++} -std=c++17 -O3 -fno-strict-aliasing -ffp-contract=off -fopenmp -fPIC -shared \
  -o "$here/_build/liboracle.so" "$here/oracle.cpp" &
p1=$!
${CXX:-g++} -std=c++17 -O3 -fno-strict-aliasing -fopenmp -fPIC -shared \
  -o "$here/_build/liboracle_time.so" "$here/oracle.cpp" &
p2=$!
wait $p1
wait $p2
