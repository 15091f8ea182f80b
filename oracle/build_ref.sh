#!/usr/bin/env bash
# Builds the UMANS reference engine, read-only from its own sources, together
# with oracle/ref_shim.cpp into oracle/_ref/libumans_ref.so.  Test
# infrastructure only: the product never links this library.
#
# The reference sources are located by $UMANS_REFERENCE (the root of a UMANS
# checkout, the directory holding src/Engine).  When it is unset or does not
# hold the sources (e.g. on a machine that only has this repository) the
# script says so and exits 0 without building anything.
#
# -ffp-contract=off keeps GCC from fusing a*b+c into an FMA; aarch64 GCC
# contracts by default, x86-64 without -mfma cannot, so this flag makes the
# oracle's arithmetic identical on both hosts.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${UMANS_REFERENCE:-}"
OUT="$HERE/_ref"
if [ -z "$REF" ]; then
  echo "UMANS_REFERENCE is not set; skipping the oracle/_ref build"
  exit 0
fi
if [ ! -d "$REF/src/Engine" ]; then
  echo "reference sources not found at \$UMANS_REFERENCE=$REF; skipping the oracle/_ref build"
  exit 0
fi
mkdir -p "$OUT"
SRC=(
  "$REF"/src/Engine/core/*.cpp
  "$REF"/src/Engine/CostFunctions/*.cpp
  "$REF"/src/Engine/tools/HelperFunctions.cpp
  "$REF"/src/Engine/tools/Polygon2D.cpp
  "$REF"/src/Engine/tools/csvwriter.cpp
  "$REF"/src/3rd-party/ORCA/ORCASolver.cpp
  "$REF"/src/3rd-party/tinyxml/tinyxml2.cpp
  "$HERE/ref_shim.cpp"
)
OBJDIR="$OUT/obj"
mkdir -p "$OBJDIR"
FLAGS=(-O2 -std=c++17 -fopenmp -ffp-contract=off -fPIC -w -I"$REF/src" -I"$REF/src/Engine")
pids=()
objs=()
for s in "${SRC[@]}"; do
  o="$OBJDIR/$(basename "${s%.cpp}").o"
  objs+=("$o")
  if [ ! -f "$o" ] || [ "$s" -nt "$o" ]; then
    g++ "${FLAGS[@]}" -c "$s" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/libumans_ref.so" "${objs[@]}"
echo "built $OUT/libumans_ref.so"
