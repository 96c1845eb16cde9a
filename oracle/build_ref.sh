#!/usr/bin/env bash
# Builds oracle/_ref/libisoref.so from the reference's own sources, where they
# lie (read-only), plus the two harness files beside this script.  Runs only
# where the reference tree exists; nothing here copies reference sources.
# Usage: oracle/build_ref.sh [reference_root]
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-/root/reference}"
LIB="$REF/isosurfaces_lib"
if [ ! -d "$LIB/isosurfaces_cuda/src" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
FLAGS=(-std=c++17 -O2 -Xcompiler -fPIC -Xcompiler -ffp-contract=off
       -gencode arch=compute_103a,code=sm_103a -w
       -I"$HERE/refshim" -I"$LIB")
nvcc "${FLAGS[@]}" -c "$HERE/ref_histogram_wrap.cu" -o "$OUT/ref_histogram_wrap.o" &
nvcc "${FLAGS[@]}" -c "$HERE/ref_approx_wrap.cu" -o "$OUT/ref_approx_wrap.o" &
nvcc "${FLAGS[@]}" -c "$LIB/isosurfaces_cuda/src/common.cu" -o "$OUT/common.o" &
wait
nvcc -shared -Xcompiler -fPIC "$OUT/ref_histogram_wrap.o" "$OUT/ref_approx_wrap.o" "$OUT/common.o" -o "$OUT/libisoref.so"
echo "built $OUT/libisoref.so"
