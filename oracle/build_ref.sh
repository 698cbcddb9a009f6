#!/usr/bin/env bash
# Compiles the reference's CPU library from its own sources, where they lie, into oracle/_ref/.
#
# TEST INFRASTRUCTURE ONLY.  The reference's CMake build needs a Fortran compiler (its project() line lists
# Fortran), which this image lacks, so the 14 library sources plus material.c are compiled directly with
# g++/gcc, as the reference would be with -fopenmp.  material.c and material.cpp go to different object
# names.  Two variants are made:
#   libref_stock.so  -- unmodified sources (CG_REL_TOL = 1e-5, ell.hpp:35)
#   libref_cg1e8.so  -- the same sources compiled against a copy of the headers in which CG_REL_TOL is
#                       1e-8 (ell.hpp:35 is an unguarded #define, so the copy is made under _ref/ at build
#                       time and never enters the repository)
# Each library also contains oracle/ref_driver.cpp, the C entry points the tests call through ctypes.
#
# Usage: oracle/build_ref.sh [reference_root]      (default: /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${MICROPP_REFERENCE:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/micropp.cpp" ]; then
  echo "reference sources not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
SRCS="material micropp micropp_c average update ell-common homogenize common solve micro3D output assembly ell instrument"
CXXFLAGS="-O3 -std=c++11 -fopenmp -fPIC -w"

build_variant() {
  local name="$1" inc="$2"
  local obj="$OUT/obj_$name"
  mkdir -p "$obj"
  local pids=()
  for s in $SRCS; do
    g++ $CXXFLAGS -I"$inc" -c "$REF/src/$s.cpp" -o "$obj/$s.o" &
    pids+=($!)
  done
  gcc -O3 -fPIC -w -I"$inc" -c "$REF/src/material.c" -o "$obj/material_c.o" &
  pids+=($!)
  g++ $CXXFLAGS -I"$inc" -I"$HERE" -c "$HERE/ref_driver.cpp" -o "$obj/ref_driver.o" &
  pids+=($!)
  for p in "${pids[@]}"; do wait "$p"; done
  g++ -shared -fopenmp -o "$OUT/libref_$name.so" "$obj"/*.o
}

build_variant stock "$REF/include"

mkdir -p "$OUT/inc_cg1e8"
cp "$REF"/include/*.hpp "$REF"/include/*.h "$OUT/inc_cg1e8/"
chmod u+w "$OUT"/inc_cg1e8/*
sed -i 's/^#define CG_REL_TOL 1.0e-5/#define CG_REL_TOL 1.0e-8/' "$OUT/inc_cg1e8/ell.hpp"
grep -q '^#define CG_REL_TOL 1.0e-8' "$OUT/inc_cg1e8/ell.hpp"
build_variant cg1e8 "$OUT/inc_cg1e8"
echo "built $OUT/libref_stock.so $OUT/libref_cg1e8.so"
