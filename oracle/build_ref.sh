#!/bin/sh
# Builds the reference-side harness from the PANSFEM2 sources where they lie
# (header-only C++; nothing is copied).  Outputs go to oracle/_ref/ only.
# Usage: oracle/build_ref.sh [path-to-PANSFEM2]   (default $PANSFEM2_REF, else /root/reference)
set -e
REF=${1:-${PANSFEM2_REF:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX=${CXX:-g++}
# parity build: no FMA contraction, so results match the reference on any host
FLAGS="-O2 -std=c++17 -fopenmp -ffp-contract=off -w"
$CXX $FLAGS -I"$REF" "$HERE/ref_driver.cpp" -o "$OUT/ref_driver"
$CXX $FLAGS "$REF/src/LinearAlgebra/Solvers/test_CG.cpp" -o "$OUT/test_CG"
for t in test_MMA test_MMA_3 test_MMA_TOY2; do
  $CXX $FLAGS "$REF/src/Optimize/Solver/$t.cpp" -o "$OUT/$t"
done
echo "built reference harness into $OUT"
