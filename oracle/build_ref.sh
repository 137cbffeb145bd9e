#!/usr/bin/env bash
# Build the reference's own hot-path sources as a CPU oracle.
# TEST INFRASTRUCTURE ONLY. Compiles the reference's Core/*.cpp where they lie
# (read-only; nothing is copied) with g++ directly (not the reference's CMake,
# which needs git metadata and downloads Eigen), against:
#   oracle/ref_include/CCPiDefines.h  project-written stand-in for the header
#                                     the reference generates from CCPiDefines.h.in
#   oracle/eigen_shim/Eigen/*         project-written subset of Eigen
# Outputs go to oracle/_ref/ only: libdvcref.so (reference classes + the C
# entry points of oracle/ref_capi.cpp) and the reference's own `dvc` and
# `strain` executables. Flags follow the reference's Release build
# (CMakeLists.txt:52, Core/CMakeLists.txt:33): -O3, OpenMP, C++11.
set -euo pipefail
REF=${DVC_REFERENCE_DIR:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
# `build_ref.sh --where`: print the reference directory (exit 3 when absent)
if [ "${1:-}" = "--where" ]; then
  [ -d "$REF/Core" ] || exit 3
  echo "$REF"
  exit 0
fi
if [ ! -d "$REF/Core" ]; then
  echo "reference sources not found at $REF; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-std=c++11 -O3 -DNDEBUG -fopenmp -fPIC -ffp-contract=off -w -I$HERE/ref_include -I$HERE/eigen_shim -I$REF/Core"
SRCS="BoundBox Cloud Point SearchParams FloatingCloud ObjectiveFunctions DataCloud InputRead Interpolate Matrix_4d Search"
pids=()
for s in $SRCS dvc strain; do
  $CXX $FLAGS -c "$REF/Core/$s.cpp" -o "$OUT/obj/$s.o" & pids+=($!)
done
$CXX $FLAGS -c "$HERE/ref_capi.cpp" -o "$OUT/obj/ref_capi.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
LIBOBJS=""
for s in $SRCS; do LIBOBJS="$LIBOBJS $OUT/obj/$s.o"; done
# -Bsymbolic-functions: the reference's calls bind to this library's own
# definitions (ref_capi.cpp's time(), for random_global's clock seed)
$CXX -shared -fopenmp -Wl,-Bsymbolic-functions -o "$OUT/libdvcref.so" $LIBOBJS "$OUT/obj/ref_capi.o"
$CXX -fopenmp -o "$OUT/dvc" "$OUT/obj/dvc.o" $LIBOBJS
$CXX -fopenmp -o "$OUT/strain" "$OUT/obj/strain.o" $LIBOBJS
echo "built $OUT/libdvcref.so $OUT/dvc $OUT/strain"
