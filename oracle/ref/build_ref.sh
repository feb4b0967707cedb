#!/bin/bash
# Builds oracle/_ref/ref_golden from the reference's own sources where they lie (read only;
# nothing is copied) plus the harness and two stand-in headers of this directory.  Host-only
# use: the reference's kernels are compiled but never launched.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REFERENCE_SRC:?set REFERENCE_SRC to the src folder of the reference checkout}"
OUT="$HERE/../_ref"
mkdir -p "$OUT"
FLAGS="-std=c++17 -rdc=true -gencode arch=compute_103a,code=sm_103a -DNDEBUG -w -I $HERE/shim -I $REF -I $REF/util"
nvcc $FLAGS -c "$REF/coredynamics.cu" -o "$OUT/coredynamics.o" &
nvcc $FLAGS -c "$REF/stats.cu" -o "$OUT/stats.o" &
nvcc $FLAGS -c "$REF/condShape.cu" -o "$OUT/condShape.o" &
nvcc $FLAGS -c "$HERE/ref_golden.cu" -o "$OUT/ref_golden.o" &
wait
nvcc -rdc=true -gencode arch=compute_103a,code=sm_103a "$OUT"/ref_golden.o "$OUT"/coredynamics.o "$OUT"/stats.o \
    "$OUT"/condShape.o -o "$OUT/ref_golden"
echo "$OUT/ref_golden"
