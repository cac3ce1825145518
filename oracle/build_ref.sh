#!/bin/sh
# Compiles the reference's own sources, unmodified and where they lie, together
# with the harness oracle/ref_harness.cpp and the project-written GLM subset,
# into oracle/_ref/ref_harness.  Test infrastructure only (pins the oracle).
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$REF/src"
if [ ! -d "$SRC" ]; then
  echo "no reference sources under $REF"
  exit 3
fi
mkdir -p "$OUT"
# the Release flags of the reference (Release/src/subdir.mk:41) plus
# -ffp-contract=off so x86-64 and aarch64 round alike
FLAGS="-std=c++14 -O3 -w -ffp-contract=off -I$HERE/glm_subset -I$SRC -I$HERE"
pids=""
for f in kernel particle kd_tree element simulation_data simulation_time gauss_integration; do
  g++ $FLAGS -c "$SRC/$f.cpp" -o "$OUT/$f.o" & pids="$pids $!"
done
for f in rings tensile rotation; do
  g++ $FLAGS -c "$SRC/benchmarks/$f.cpp" -o "$OUT/$f.o" & pids="$pids $!"
done
g++ $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" & pids="$pids $!"
for p in $pids; do wait $p; done
g++ -o "$OUT/ref_harness" "$OUT"/*.o
echo "built $OUT/ref_harness"
