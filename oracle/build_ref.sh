#!/usr/bin/env bash
# Builds oracle/_ref/libsgref.so: the reference's own hot-path headers,
# unmodified, compiled against this folder's shims. TEST INFRASTRUCTURE
# ONLY. Needs the reference sources: $SG_REF, by default a checkout named
# `reference` beside this repository; without them it exits 0 and builds
# nothing (the GPU machine has no copy).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${SG_REF:-$here/../../reference}"
if [ ! -d "$ref/singularity-eos" ]; then
  echo "build_ref: reference sources not found at $ref; skipping" >&2
  exit 0
fi
mkdir -p "$here/_ref"
g++ -std=c++17 -O2 -fPIC -shared -fopenmp -ffp-contract=off -fno-lifetime-dse -DNDEBUG \
  -DSINGULARITY_USE_SPINER -DSINGULARITY_USE_SPINER_WITH_HDF5 \
  -DSINGULARITY_USE_HELMHOLTZ -DSINGULARITY_BUILD_CLOSURE \
  -I "$here/shims" -I "$ref" \
  "$here/sgref.cpp" -o "$here/_ref/libsgref.so.tmp"
mv "$here/_ref/libsgref.so.tmp" "$here/_ref/libsgref.so"
echo "build_ref: built $here/_ref/libsgref.so"
