#!/usr/bin/env bash
# ORACLE — test infrastructure only. Compiles the reference's own CPU solver
# (domain/water_state/src/water_state.cpp and the few core/ sources it links) straight from the
# reference's source tree, with the reference's no-contraction policy, into
# oracle/_ref/libwsref.so behind oracle/ref_shim.cpp. Nothing is copied out of the reference; the
# reference's own build system (CMake, FetchContent) is not run.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]
#
# The root is the argument, else $WL_REFERENCE_ROOT, else the place this recipe reads the
# reference's sources from on the build machine (below). The root it built from is recorded in
# oracle/_ref/reference_root, so that the tests and fixture generators that read the reference's
# headers find them without naming a path. Exits 0 without building when the reference's sources
# are absent (a machine that only runs the tests has none).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${WL_REFERENCE_ROOT:-/root/reference}}"
OUT="$HERE/_ref"
if [[ ! -f "$REF/domain/water_state/src/water_state.cpp" ]]; then
  echo "build_ref: no reference sources at $REF; skipped"
  exit 0
fi
mkdir -p "$OUT"
INC=()
for d in "$REF"/core/*/include "$REF"/domain/water_state/include; do INC+=("-I$d"); done
SRC=(
  "$REF/domain/water_state/src/water_state.cpp"
  "$REF/core/base/src/assert.cpp"
  "$REF/core/memory/src/memory.cpp"
  "$REF/core/memory/src/arena.cpp"
  "$REF/core/jobs/src/job_system.cpp"
  "$REF"/core/platform/src/*.cpp
  "$REF"/core/profiling/src/*.cpp
  "$REF"/core/json/src/*.cpp
  "$HERE/ref_shim.cpp"
)
FLAGS=(-std=c++20 -O2 -fPIC -ffp-contract=off
       -DENGINE_FP_CONTRACTION=0 -DENGINE_MEMORY_TRACKING=0 -DENGINE_PROFILING=0)
OBJ=()
pids=()
for s in "${SRC[@]}"; do
  o="$OUT/$(basename "${s%.cpp}").o"
  OBJ+=("$o")
  g++ "${FLAGS[@]}" "${INC[@]}" -c "$s" -o "$o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libwsref.so" "${OBJ[@]}" -lpthread
rm -f "${OBJ[@]}"
printf '%s\n' "$REF" > "$OUT/reference_root"
echo "build_ref: $OUT/libwsref.so"
