#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.  Compiles the reference's host-side loader and
# virtual-graph code from the sources where they lie (read-only) together with
# the two dump drivers in this folder.  Outputs go to oracle/_ref/ only, which
# git ignores.  Needs the reference checkout; skips quietly without it.
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
