#!/usr/bin/env bash
# Compile the pin driver (oracle/ref_pin.cpp) against the reference's own sources
# where they lie in the reference tree.  Outputs only into oracle/_ref/.
#   ref_pin_f64 : -DUSE_DOUBLE (scalar CubicKernel, Eigen CG + BlockJacobiPreconditioner3D)
#   ref_pin_f32 : -DUSE_AVX    (scalar CubicKernel and CubicKernel_AVX in float)
# The reference's own build system is not used: its CMake project needs external
# projects (CompactNSearch, GenericParameters, Discregrid) that are not in the tree.
# Only the self-contained pieces are compiled: SPlisHSPlasH/SPHKernels.cpp and the
# header-only SPlisHSPlasH/Utilities/MatrixFreeSolver.h with the vendored Eigen.
set -euo pipefail
REF=${SPH_REFERENCE_ROOT:-/root/reference}
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/SPlisHSPlasH/SPHKernels.cpp" ]; then
  echo "reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
INC="-I$REF -I$REF/SPlisHSPlasH -I$REF/extern/eigen -I$HERE"
$CXX -O2 -std=c++17 -ffp-contract=off -DUSE_DOUBLE $INC -x c++ "$HERE/sph_oracle.c" -x none \
    "$HERE/ref_pin.cpp" "$REF/SPlisHSPlasH/SPHKernels.cpp" -o "$OUT/ref_pin_f64" -fopenmp -w
if [ "$(uname -m)" = "x86_64" ]; then
  $CXX -O2 -std=c++17 -ffp-contract=off -DUSE_AVX -mavx2 -mfma $INC \
      "$HERE/ref_pin.cpp" "$REF/SPlisHSPlasH/SPHKernels.cpp" -o "$OUT/ref_pin_f32" -w
fi
echo "built into $OUT"
