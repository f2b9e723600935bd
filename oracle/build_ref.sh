#!/usr/bin/env bash
# Compiles the reference's kernel header for the CPU (test infrastructure).
# Usage: build_ref.sh <reference checkout>   (or SGDLM_REFERENCE=<checkout>)
# Reads the reference sources where they lie; writes only oracle/_ref/.
# The macro values are those of the reference's build (rSGDLM/src/Makevars.in:1).
# Exit status 2: no reference checkout given or found there.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT_REF="${1:-${SGDLM_REFERENCE:-}}"
if [ -z "$ROOT_REF" ]; then
  echo "usage: build_ref.sh <reference checkout> (or set SGDLM_REFERENCE)" >&2
  exit 2
fi
REF="$ROOT_REF/rSGDLM/src"
if [ ! -f "$REF/kernel_functions.cuh" ]; then
  echo "reference sources not found at $REF" >&2
  exit 2
fi
mkdir -p "$HERE/_ref"
g++ -O1 -std=c++17 -fPIC -shared \
  -I "$HERE/ref_shim" -I "$REF" \
  -DTHREADS_PER_BLOCK=512 -DOPTIM_PRECISION=0.000001 -DOPTIM_MAX_ITER=50 -DGAMMA_LOOPS=2 \
  "$HERE/ref_driver.cpp" -o "$HERE/_ref/libref_kernels.so"
echo "$HERE/_ref/libref_kernels.so"
