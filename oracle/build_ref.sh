#!/usr/bin/env bash
# Builds the DROPS reference implementation of the TraceFEM path, read in place
# from its source tree, together with oracle/ref_harness.cpp, into
# oracle/_ref/ref_harness.  Test infrastructure only: it runs where the
# reference sources exist and is never part of the product.
#
#   oracle/build_ref.sh [REFERENCE_SRC_DIR]      (default /root/reference/src)
#
# Flags: -O2 -fopenmp, no --fast-math (the reference's default DEBUG-less
# build), -include cstring (geom/signtraits.h) and -include iomanip
# (misc/progressaccu.cpp) and -include memory (levelset/levelsetmapper.h names
# std::unique_ptr without including <memory>) for headers the sources assume, and oracle/refshim/ on the
# include path in place of Boost.PropertyTree.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="${1:-/root/reference/src}"
OUT="$HERE/_ref"
OBJ="$OUT/obj"
mkdir -p "$OBJ"
CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O2 -fopenmp -ffp-contract=off -w -include cstring -include iomanip -include memory -I "$SRC" -I "$HERE/refshim")
UNITS=(
  geom/topo.cpp geom/simplex.cpp geom/multigrid.cpp geom/builder.cpp geom/boundary.cpp
  geom/principallattice.cpp geom/reftetracut.cpp geom/subtriangulation.cpp geom/locator.cpp
  geom/deformation.cpp
  num/discretize.cpp num/quadrature.cpp num/unknowns.cpp num/fe.cpp num/interfacePatch.cpp num/bndData.cpp
  num/gradient_recovery.cpp levelset/levelsetmapper.cpp
  misc/utils.cpp misc/problem.cpp misc/params.cpp misc/scopetimer.cpp
  surfactant/ifacetransp.cpp
  levelset/adaptriang.cpp levelset/marking_strategy.cpp
  levelset/levelset.cpp levelset/surfacetension.cpp levelset/fastmarch.cpp levelset/volume_adjustment.cpp
  out/vtkOut.cpp out/ensightOut.cpp misc/progressaccu.cpp misc/base64.cpp
)
compile() {
  local u="$1"; local o="$OBJ/$(echo "$u" | tr '/' '_').o"
  if [[ ! -f "$o" || "$SRC/$u" -nt "$o" ]]; then "$CXX" "${FLAGS[@]}" -c "$SRC/$u" -o "$o"; fi
}
export -f compile; export SRC OBJ CXX; export FLAGS_STR="${FLAGS[*]}"
pids=()
for u in "${UNITS[@]}"; do compile "$u" & pids+=($!); 
  if (( ${#pids[@]} >= $(nproc) )); then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" "${FLAGS[@]}" -fno-access-control -c "$HERE/ref_harness.cpp" -o "$OBJ/ref_harness.o"
"$CXX" -fopenmp -o "$OUT/ref_harness" "$OBJ"/*.o
echo "built $OUT/ref_harness"

# The DROPS drop-in shim (drops_gb300/adapter) compiled against the reference's
# own headers, and its check driver, linked with the reference objects and
# libtracefem (built first by drops_gb300/build.py).
REPO="$(cd "$HERE/.." && pwd)"
LIBDIR="$REPO/drops_gb300/_lib"
if [[ -f "$LIBDIR/libtracefem.so" ]]; then
  AOBJ="$OUT/adapter_obj"
  mkdir -p "$AOBJ"
  AFLAGS=("${FLAGS[@]}" -I "$REPO/include" -I "$REPO/drops_gb300/adapter")
  "$CXX" "${AFLAGS[@]}" -c "$REPO/drops_gb300/adapter/tracefem_drops.cpp" -o "$AOBJ/tracefem_drops.o"
  "$CXX" "${AFLAGS[@]}" -c "$HERE/adapter_check.cpp" -o "$AOBJ/adapter_check.o"
  REFOBJ=()
  for o in "$OBJ"/*.o; do [[ "$(basename "$o")" == ref_harness.o ]] || REFOBJ+=("$o"); done
  CUDALIB="${CUDA_HOME:-/usr/local/cuda}/lib64"
  "$CXX" -fopenmp -o "$OUT/adapter_check" "$AOBJ/adapter_check.o" "$AOBJ/tracefem_drops.o" "${REFOBJ[@]}" \
    -L "$LIBDIR" -ltracefem -Wl,-rpath,"$LIBDIR" -L "$CUDALIB" -Wl,-rpath,"$CUDALIB"
  echo "built $OUT/adapter_check"
fi
