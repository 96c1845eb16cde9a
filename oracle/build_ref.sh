#!/usr/bin/env bash
# Builds the reference checkers under oracle/_ref/ from the reference's own
# sources, where they lie (read-only), plus the harness files beside this
# script; nothing here copies reference sources.
#   libisoref.so         host functions of JointHistogram.cu and
#                        IsosurfaceApproximation.cu (CPU golden vectors)
#   ref_histogram.cubin  device code of JointHistogram.cu (the reference's own
#                        histogram kernel, run on a GPU by oracle/refgpu.py),
#                        compiled with nvcc's default flags as the reference's
#                        CMake build does (no -fmad or precision flags)
#   ref_mc.cubin         device code of MarchingCube.cu (the reference's own
#                        marching-cubes kernels) with its lookup tables as
#                        device arrays (oracle/ref_mc_wrap.cu), nvcc defaults;
#                        refshim_mc/refshim_texture.h stands in for the
#                        texture references CUDA 13 no longer has
#   ref_bvh.cubin        device code of BVH.cu (the reference's own LBVH build
#                        and traversal) with oracle/ref_bvh_wrap.cu, nvcc
#                        defaults
#   ref_approx.cubin     device code of IsosurfaceApproximation.cu (the
#                        reference's voxel-approximation kernel), nvcc defaults
# Runs only where the reference tree exists.
# Usage: oracle/build_ref.sh [reference_root]   (default: $ISO_REFERENCE_ROOT,
#        else /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${ISO_REFERENCE_ROOT:-/root/reference}}"
LIB="$REF/isosurfaces_lib"
if [ ! -d "$LIB/isosurfaces_cuda/src" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
ARCH=(-gencode arch=compute_103a,code=sm_103a)
FLAGS=(-std=c++17 -O2 -Xcompiler -fPIC -Xcompiler -ffp-contract=off "${ARCH[@]}" -w
       -I"$HERE/refshim" -I"$LIB")
nvcc "${FLAGS[@]}" -c "$HERE/ref_histogram_wrap.cu" -o "$OUT/ref_histogram_wrap.o" &
nvcc "${FLAGS[@]}" -c "$HERE/ref_approx_wrap.cu" -o "$OUT/ref_approx_wrap.o" &
nvcc "${FLAGS[@]}" -c "$LIB/isosurfaces_cuda/src/common.cu" -o "$OUT/common.o" &
nvcc -std=c++17 -cubin "${ARCH[@]}" -w -I"$HERE/refshim" -I"$LIB" \
  "$LIB/isosurfaces_cuda/src/JointHistogram.cu" -o "$OUT/ref_histogram.cubin" &
nvcc -std=c++17 -cubin "${ARCH[@]}" -w -include "$HERE/refshim_mc/refshim_texture.h" -I"$HERE/refshim" -I"$LIB" \
  "$HERE/ref_mc_wrap.cu" -o "$OUT/ref_mc.cubin" &
nvcc -std=c++17 -cubin "${ARCH[@]}" -w -I"$HERE/refshim" -I"$LIB" \
  "$HERE/ref_bvh_wrap.cu" -o "$OUT/ref_bvh.cubin" &
nvcc -std=c++17 -cubin "${ARCH[@]}" -w -I"$HERE/refshim" -I"$LIB" \
  "$LIB/isosurfaces_cuda/src/IsosurfaceApproximation.cu" -o "$OUT/ref_approx.cubin" &
wait
nvcc -shared -Xcompiler -fPIC "$OUT/ref_histogram_wrap.o" "$OUT/ref_approx_wrap.o" "$OUT/common.o" -o "$OUT/libisoref.so"
# where the sources were found, for the CPU tests that read the reference's
# tables directly (oracle.reference_root())
echo "$REF" > "$OUT/reference_root.txt"
echo "built $OUT/libisoref.so and the reference cubins (histogram, marching cubes, LBVH, approximation)"
