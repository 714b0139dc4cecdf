#!/usr/bin/env bash
# Build recipe for the reference side of the parity checker (test infrastructure only).
#
# 1. fdtdrav_sm103a.cubin: the reference's own kernels (fdtdrav.h), compiled from the reference
#    checkout where it lies, for sm_103a. Needs the checkout, so it is built only where the
#    checkout exists; the cubin is host-independent and is carried to the GPU machine.
# 2. librefharness.so: our host runner that loads that cubin (built wherever CUDA is present).
#
# Outputs go only to oracle/_ref/. Usage: oracle/build_ref.sh [reference_dir]; the reference
# checkout is the argument, else $FDTD_REFERENCE_DIR; without either only the runner is built.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${FDTD_REFERENCE_DIR:-}}"
OUT="$HERE/_ref"
NVCC="${NVCC:-nvcc}"
mkdir -p "$OUT"

if [ -n "$REF" ] && [ -f "$REF/fdtdrav.h" ]; then
  "$NVCC" -cubin -O3 -gencode arch=compute_103a,code=sm_103a -I"$REF" \
      -o "$OUT/fdtdrav_sm103a.cubin" "$HERE/ref_harness/ref_kernels.cu"
fi

"$NVCC" -O2 -shared -Xcompiler -fPIC -o "$OUT/librefharness.so" "$HERE/ref_harness/ref_runner.cu"
