#!/usr/bin/env bash
# Test infrastructure.  Compiles the reference's own DFSPH time step from its sources
# where they lie in the reference tree (SPH_REFERENCE_ROOT, or ../reference next to
# this repository), against the stand-ins in oracle/shims/ for the external projects
# that the tree does not hold (CompactNSearch, GenericParameters, Discregrid).
# Outputs go only into oracle/_ref/:
#   libref_f64.so : -DUSE_DOUBLE, scalar code paths, the oracle pin (ref_driver.cpp)
#   libref_f32.so : -DUSE_AVX -DUSE_PERFORMANCE_OPTIMIZATION, the reference's FP32 AVX
#                   path as its CMake release build configures it (x86-64 hosts only)
#   ref_pin_f64 / ref_pin_f32 : kernel values and Eigen CG (ref_pin.cpp)
# The reference's CMake project is not used: it fetches those external projects over
# the network.  Two headers the reference relies on transitively (<cfloat>, <memory>)
# are force-included because this compiler's standard library no longer pulls them in.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF=${SPH_REFERENCE_ROOT:-"$HERE/../../reference"}
OUT="$HERE/_ref"
if [ ! -f "$REF/SPlisHSPlasH/TimeStep.cpp" ]; then
  echo "reference tree not found at $REF (set SPH_REFERENCE_ROOT); skipping" >&2
  exit 0
fi
REF="$(cd "$REF" && pwd)"
mkdir -p "$OUT"
CXX=${CXX:-g++}
JOBS=${JOBS:-$(nproc)}

# the reference's library sources (SPlisHSPlasH/CMakeLists.txt), less the mesh-sampling
# utilities that need a real Discregrid (SDFFunctions, VolumeSampling); the library also
# links two vendored projects of the tree, extern/md5 and extern/tinyexpr
SOURCES=$(cd "$REF" && ls SPlisHSPlasH/*.cpp SPlisHSPlasH/DFSPH/*.cpp SPlisHSPlasH/WCSPH/*.cpp \
  SPlisHSPlasH/PCISPH/*.cpp SPlisHSPlasH/PBF/*.cpp SPlisHSPlasH/IISPH/*.cpp SPlisHSPlasH/PF/*.cpp \
  SPlisHSPlasH/ICSPH/*.cpp SPlisHSPlasH/Viscosity/*.cpp SPlisHSPlasH/Drag/*.cpp SPlisHSPlasH/Elasticity/*.cpp \
  SPlisHSPlasH/SurfaceTension/*.cpp SPlisHSPlasH/Vorticity/*.cpp SPlisHSPlasH/Utilities/*.cpp \
  | grep -v -e 'Utilities/SDFFunctions.cpp' -e 'Utilities/VolumeSampling.cpp')
INC="-include cfloat -include memory -I$HERE/shims -I$REF -I$REF/extern/eigen -I$REF/extern"

build_lib() {   # name, flags...
  local name=$1; shift
  local flags="$*"
  local obj="$OUT/obj_$name"
  mkdir -p "$obj"
  export CXX INC REF obj flags
  # shellcheck disable=SC2016
  printf '%s\n' $SOURCES | xargs -P "$JOBS" -I{} bash -c \
    'o="$obj/$(echo {} | tr / _).o"; [ "$o" -nt "$REF/{}" ] || $CXX -std=c++17 -fPIC -fopenmp -w $flags $INC -c "$REF/{}" -o "$o"'
  $CXX -std=c++17 -fPIC -fopenmp -w $flags $INC -c "$HERE/ref_driver.cpp" -o "$obj/ref_driver.o"
  # vendored third-party code the library links (extern/md5, extern/tinyexpr)
  $CXX -std=c++17 -fPIC -w -O2 -I"$REF/extern/md5" -c "$REF/extern/md5/md5.cpp" -o "$obj/extern_md5.o"
  ${CC:-gcc} -fPIC -w -O2 -c "$REF/extern/tinyexpr/tinyexpr.c" -o "$obj/extern_tinyexpr.o"
  # the oracle's grid evaluation behind ref_driver.cpp's Discregrid grid (volume maps), with
  # the oracle's kernel functions it uses (FP64)
  ${CC:-gcc} -std=c11 -fPIC -fopenmp -w -O2 -ffp-contract=off -DORC_REAL=double -c "$HERE/vmap.c" -o "$obj/oracle_vmap.o"
  ${CC:-gcc} -std=c11 -fPIC -fopenmp -w -O2 -ffp-contract=off -DORC_REAL=double -c "$HERE/sph_oracle.c" -o "$obj/oracle_sph.o"
  $CXX -shared -fopenmp -Wl,--no-undefined -o "$OUT/lib$name.so.tmp" "$obj"/*.o -lm
  mv "$OUT/lib$name.so.tmp" "$OUT/lib$name.so"
}

build_lib ref_f64 -O2 -ffp-contract=off -DUSE_DOUBLE
if [ "$(uname -m)" = "x86_64" ]; then
  build_lib ref_f32 -O3 -DNDEBUG -march=native -mavx2 -mfma -DUSE_AVX -DUSE_PERFORMANCE_OPTIMIZATION
fi

# kernel values and Eigen CG pins (ref_pin.cpp) against the oracle restatement
$CXX -O2 -std=c++17 -ffp-contract=off -DUSE_DOUBLE -I"$REF" -I"$REF/SPlisHSPlasH" -I"$REF/extern/eigen" -I"$HERE" \
    -x c++ "$HERE/sph_oracle.c" -x c++ "$HERE/vmap.c" -x none \
    "$HERE/ref_pin.cpp" "$REF/SPlisHSPlasH/SPHKernels.cpp" -o "$OUT/ref_pin_f64" -fopenmp -w
if [ "$(uname -m)" = "x86_64" ]; then
  $CXX -O2 -std=c++17 -ffp-contract=off -DUSE_AVX -mavx2 -mfma -I"$REF" -I"$REF/SPlisHSPlasH" -I"$REF/extern/eigen" \
      -I"$HERE" "$HERE/ref_pin.cpp" "$REF/SPlisHSPlasH/SPHKernels.cpp" -o "$OUT/ref_pin_f32" -w
fi
echo "built into $OUT"
