#!/usr/bin/env bash
# Builds the reference FLIP engine (jklae/FLIPEngine3D, src/engine/*.cpp) from
# its read-only sources, plus oracle/ref/ref_harness.cpp, into
# oracle/_ref/libflipref.so.  Test-only: the library is the checker the C++
# restatement in oracle/ is pinned against; nothing in the product loads it.
#
# The reference ships no build for its engine alone (its CMake file builds the
# Win32 viewer), so the engine's translation units are compiled directly.
# GCC 13 needs <limits> force-included (src/engine/trianglemesh.cpp uses
# std::numeric_limits without including it).  -ffp-contract=off keeps float
# arithmetic unfused on every host, matching an x86-64 -O2 build.
set -euo pipefail
REF="${FLIP_REFERENCE_ROOT:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/src/engine"
if [ ! -d "$SRC" ]; then
  echo "reference sources not found at $SRC; oracle/_ref not built" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
CXXFLAGS="-std=c++14 -O2 -pthread -fPIC -include limits -ffp-contract=off -w"
JOBS="$(nproc)"

objs=()
pids=()
for f in "$SRC"/*.cpp; do
  o="$OUT/obj/$(basename "${f%.cpp}").o"
  objs+=("$o")
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
    g++ $CXXFLAGS -I"$SRC" -c "$f" -o "$o" &
    pids+=($!)
    if [ "${#pids[@]}" -ge "$JOBS" ]; then
      wait "${pids[0]}"; pids=("${pids[@]:1}")
    fi
  fi
done
for p in "${pids[@]}"; do wait "$p"; done

g++ $CXXFLAGS -I"$SRC" -c "$HERE/ref/ref_harness.cpp" -o "$OUT/ref_harness.o"
g++ -shared -pthread -o "$OUT/libflipref.so" "${objs[@]}" "$OUT/ref_harness.o"
echo "built $OUT/libflipref.so"
