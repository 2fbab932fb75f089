#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# No -march=native and no fused multiply-add, so that x86-64 and aarch64 hosts
# produce bit-identical results.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CXX:-g++} -std=c++17 -O3 -fno-strict-aliasing -ffp-contract=off -fopenmp -fPIC -shared \
  -o "$here/_build/liboracle.so" "$here/oracle.cpp"
