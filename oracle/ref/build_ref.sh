#!/bin/sh
# Build oracle/_ref/libflare_ref.so from the reference's own sources, compiled
# where they lie in the reference tree: the L0 math (radial.cpp, cutoffs.cpp,
# y_grad.cpp, descriptors/wigner3j.cpp), Structure (structure.cpp), B2, B3 and
# DescriptorValues (descriptors/b2.cpp, b3.cpp, descriptor.cpp), the
# NormalizedDotProduct kernel (kernels/kernel.cpp, normalized_dot_product.cpp),
# the sparse GP (bffs/sparse_gp.cpp)
# and the pair style's per-atom math (lammps_plugins/lammps_descriptor.cpp),
# plus oracle/ref/ref_shim*.cpp.  Only the small Eigen and nlohmann_json
# stand-ins in oracle/ref/stub are added; no reference file is copied or
# modified.
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
  -I"$HERE/stub" -I"$SRC" -I"$SRC/descriptors" -I"$SRC/kernels" -I"$SRC/bffs" \
  -I"$REF/lammps_plugins" \
  "$SRC/radial.cpp" "$SRC/cutoffs.cpp" "$SRC/y_grad.cpp" \
  "$SRC/descriptors/wigner3j.cpp" "$REF/lammps_plugins/lammps_descriptor.cpp" \
  "$SRC/structure.cpp" "$SRC/descriptors/descriptor.cpp" "$SRC/descriptors/b2.cpp" \
  "$SRC/descriptors/b3.cpp" "$SRC/bffs/sparse_gp.cpp" \
  "$SRC/kernels/kernel.cpp" "$SRC/kernels/normalized_dot_product.cpp" \
  "$HERE/ref_shim.cpp" "$HERE/ref_shim_struc.cpp" "$HERE/ref_shim_sgp.cpp" \
  -o "$OUT/libflare_ref.so"
echo "built $OUT/libflare_ref.so"
