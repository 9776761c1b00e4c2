#!/usr/bin/env bash
# Build the reference's own hot-path C++ (read in place from the reference tree,
# never copied) plus oracle/ref_shim.cpp and oracle/ref_capi.cpp into
# oracle/_ref/libtopopt_ref.so.  Test infrastructure: a checker and the timed CPU
# baseline, never linked into the product.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default $TOPOPT_REFERENCE_ROOT, else /root/reference)
# Skips with exit 0 when the reference tree is absent (e.g. on a GPU machine).
set -euo pipefail
REF="${1:-${TOPOPT_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/core/src" ]; then
  echo "build_ref: reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
CORE="$REF/core"
# The Eigen-free translation units of the path and the base files they pull in.
SRCS="fea/hex_element fea/matfree fea/recycle simp/simp voxel/voxelize simp/observability orient/orient settings/report settings/gate_diagnosis_report io/design_store io/fields
      simp/mma_joint simp/semdot fea/lattice_material mesh/mesh fea/lattice"
CXXFLAGS="-std=c++17 -O3 -fPIC -I$CORE/include -I$CORE/src"
pids=()
for s in $SRCS; do
  o="$OUT/obj/$(echo "$s" | tr / _).o"
  if [ ! -f "$o" ] || [ "$CORE/src/$s.cpp" -nt "$o" ]; then
    g++ $CXXFLAGS -c "$CORE/src/$s.cpp" -o "$o" &
    pids+=($!)
  fi
done
g++ $CXXFLAGS -c "$HERE/ref_shim.cpp" -o "$OUT/obj/ref_shim.o" &
pids+=($!)
g++ $CXXFLAGS -c "$HERE/ref_capi.cpp" -o "$OUT/obj/ref_capi.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libtopopt_ref.so" "$OUT"/obj/*.o -lpthread -Wl,--no-undefined
echo "build_ref: $OUT/libtopopt_ref.so"
