#!/bin/bash
# Compiles the reference's GPU kernels, from its own sources where they lie (read only; nothing
# is copied), into one device-only module oracle/_ref/ref_kernels.cubin for sm_103a, together
# with the helper kernels of oracle/ref/ref_kernels_unity.cu.  Checker only: the module is
# loaded by oracle/ref/ref_kernel_runner.cu through the CUDA driver API to produce golden
# vectors (tests/golden/make_ref_kernel_golden.py); the product never uses it.
#   REFERENCE_SRC=<reference checkout>/src bash oracle/ref/build_ref_kernels.sh
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REFERENCE_SRC:?set REFERENCE_SRC to the src folder of the reference checkout}"
OUT="$HERE/../_ref"
mkdir -p "$OUT"
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -DNDEBUG -w \
    -I "$HERE/shim" -I "$REF" -I "$REF/util" -o "$OUT/ref_kernels.cubin" "$HERE/ref_kernels_unity.cu"
echo "$OUT/ref_kernels.cubin"
