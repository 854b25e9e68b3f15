#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.  Needs the reference checkout; skips quietly
# without it.  Outputs go to oracle/_ref/ only, which git ignores.
#   1. Compiles the reference's host-side loader and virtual-graph code from
#      the sources where they lie (read-only) together with the two dump
#      drivers in this folder (golden loader fixtures).
#   2. Copies the sources of the reference's seven GPU decomposition drivers,
#      unmodified, into oracle/_ref/src, so that they travel with the working
#      tree to a GPU machine (which has no reference checkout); oracle/ref_gpu.py
#      compiles them there with nvcc for sm_103a.
set -euo pipefail
REF="${PICO_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/index2core/shared" ]; then
  echo "build_ref: reference sources not present; skipped"
  exit 0
fi
mkdir -p "$OUT"
g++ -O2 -std=c++14 -w -I"$REF/index2core/shared" "$HERE/ref_dump_coo.cpp" \
    "$REF/index2core/shared/graph.cpp" "$REF/index2core/shared/virtual_graph.cpp" \
    -o "$OUT/ref_dump_coo"
g++ -O2 -std=c++14 -w -fopenmp -I"$REF/peel/inc" "$HERE/ref_dump_csr.cpp" \
    "$REF/peel/src/graph.cpp" -o "$OUT/ref_dump_csr"
echo "build_ref: built $OUT/ref_dump_coo $OUT/ref_dump_csr"
SRC="$OUT/src"
mkdir -p "$SRC/index2core/shared" "$SRC/peel/shared" "$SRC/peel/src" "$SRC/peel/inc"
for f in HistoCore.cu CntCore.cu NbrCore.cu; do cp -p "$REF/index2core/$f" "$SRC/index2core/"; done
cp -p "$REF"/index2core/shared/*.cpp "$REF"/index2core/shared/*.h "$REF"/index2core/shared/*.cuh "$SRC/index2core/shared/"
for f in peelone.cu gppeel.cu; do cp -p "$REF/peel/$f" "$SRC/peel/"; done
cp -p "$REF"/peel/shared/*.cpp "$REF"/peel/shared/*.h "$REF"/peel/shared/*.cuh "$SRC/peel/shared/"
cp -p "$REF"/peel/src/* "$SRC/peel/src/"
cp -p "$REF"/peel/inc/* "$SRC/peel/inc/"
echo "build_ref: copied the GPU driver sources to $SRC"
