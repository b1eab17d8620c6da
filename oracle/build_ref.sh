#!/usr/bin/env bash
# Builds oracle/_ref/ from the reference's own sources, where they lie.
# TEST INFRASTRUCTURE ONLY; needs the reference source tree, named by the
# REF_DIR environment variable (required; nothing is built without it).
# Outputs go to oracle/_ref/ and nowhere else; the reference tree is only read.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:?set REF_DIR to the reference source tree}"
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/graph.h" ]; then
  echo "reference tree not found at $REF_DIR; oracle/_ref not built" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
# The graph files the reference's GPU search reads are written by `song build`
# (build_graph.sh:9), whose host code nvcc hands to g++ as -std=c++11 -O3 with
# no -march (Makefile:10-18): on x86-64 that target has no FMA, so the float
# norm sums of the cosine distance (data.h:53-58) are not contracted.
# -ffp-contract=off pins that behaviour on any host.  (song.cpu's -march=native,
# Makefile:7-8, lets g++ contract them on FMA hosts; that build is not used.)
FLAGS="-std=c++11 -O3 -ffp-contract=off -fPIC -shared -w -I$REF_DIR"
# degree-32 graph: config.h as shipped (FIXED_DEGREE 31, SHIFT 5, SEARCH_DEGREE 15)
$CXX $FLAGS "$HERE/ref_harness.cpp" -o "$OUT/libsongref_s5.so" &
# degree-16 graph: FIXED_DEGREE 15, SHIFT 4, SEARCH_DEGREE 7
$CXX $FLAGS -DREF_FIXED_DEGREE=15 -DREF_SHIFT=4 -DREF_SEARCH_DEGREE=7 \
  "$HERE/ref_harness.cpp" -o "$OUT/libsongref_s4.so" &
wait
echo "built $OUT/libsongref_s5.so $OUT/libsongref_s4.so"
