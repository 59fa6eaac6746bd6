#!/usr/bin/env bash
# Builds oracle/_build/libsgport.so from oracle/port/sgport.cpp (this
# project's restatement of the reference algorithms; TEST INFRASTRUCTURE
# ONLY). Portable C++17, no architecture-specific flags, no FP contraction.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
g++ -std=c++17 -O2 -fPIC -shared -fopenmp -ffp-contract=off \
  "$here/port/sgport.cpp" -o "$here/_build/libsgport.so.tmp"
mv "$here/_build/libsgport.so.tmp" "$here/_build/libsgport.so"
echo "build_port: built $here/_build/libsgport.so"
