#!/bin/sh
# Build oracle/_ref/libflare_ref.so from the reference's own L0 math sources
# (radial.cpp, cutoffs.cpp, y_grad.cpp, descriptors/wigner3j.cpp) and its
# per-atom pair-style math (lammps_plugins/lammps_descriptor.cpp), compiled
# where they lie in the reference tree, plus oracle/ref/ref_shim.cpp.  Only the
# small Eigen stand-in in oracle/ref/stub is added; no reference file is copied
# or modified.
# Usage: oracle/ref/build_ref.sh [reference_root]
#        (default: $FLARE_PP_REFERENCE, else /root/reference)
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${FLARE_PP_REFERENCE:-/root/reference}}"
SRC="$REF/src/flare_pp"
OUT="$HERE/../_ref"
if [ ! -f "$SRC/radial.cpp" ]; then
  echo "reference sources not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off \
  -I"$HERE/stub" -I"$SRC" -I"$SRC/descriptors" -I"$REF/lammps_plugins" \
  "$SRC/radial.cpp" "$SRC/cutoffs.cpp" "$SRC/y_grad.cpp" \
  "$SRC/descriptors/wigner3j.cpp" "$REF/lammps_plugins/lammps_descriptor.cpp" \
  "$HERE/ref_shim.cpp" -o "$OUT/libflare_ref.so"
echo "built $OUT/libflare_ref.so"
