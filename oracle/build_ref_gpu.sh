#!/usr/bin/env bash
# Rebuilds the reference's GPU search kernel (warp_astar_accelerator.h:41-341)
# for sm_100, one cubin per (metric, dim, pq_size), into oracle/_ref/.
# TEST INFRASTRUCTURE ONLY; needs the reference source tree, named by the
# REF_DIR environment variable (required; nothing is built without it).
#
# The reference fixes TOPK (= pq_size) and DIM at compile time with its
# template step (generate_template.sh:16-34, fill_parameters.sh:35-53: sed of
# the "#define TOPK" / "#define DIM" lines).  This script does the same two
# substitutions on a scratch copy under /tmp and builds with the reference's
# flags (Makefile:10-18: -O3, -D$(DISTTYPE) -D__ENABLE_FIXHASH
# -D__ENABLE_VISITED_DEL), for -gencode arch=compute_100,code=sm_100.  Two
# builds per case: __ENABLE_MEASURE as shipped (warp_astar_accelerator.h:32)
# and with that line removed.  The reference tree itself is only read.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:?set REF_DIR to the reference source tree}"
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/warp_astar_accelerator.h" ]; then
  echo "reference tree not found at $REF_DIR; reference cubins not built" >&2
  exit 0
fi
NVCC="${NVCC:-nvcc}"
SCRATCH="$(mktemp -d /tmp/song_ref_gpu.XXXXXX)"
trap 'rm -rf "$SCRATCH"' EXIT
mkdir -p "$OUT"
# cases: metric:dim:pq
CASES="${CASES:-cos:16:10 cos:16:50 cos:16:100 l2:32:10 l2:32:50 l2:32:100 ip:24:10 ip:24:50 ip:24:100 cos:26:10 cos:26:50 cos:26:100 l2:128:100 l2:128:200 l2:128:400 l2:128:600 l2:128:800 l2:128:1000}"
build_one() {
  local metric=$1 dim=$2 pq=$3 measure=$4
  local dir="$SCRATCH/${metric}_${dim}_${pq}_${measure}"
  mkdir -p "$dir"
  cp "$REF_DIR"/*.h "$dir"/
  sed -i -e "s/#define TOPK.*/#define TOPK $pq/" "$dir/astar_accelerator.h"
  sed -i -e "s/#define DIM.*/#define DIM $dim/" "$dir/warp_astar_accelerator.h"
  if [ "$measure" = "nomeasure" ]; then
    sed -i -e "s/^#define __ENABLE_MEASURE$//" "$dir/warp_astar_accelerator.h"
  fi
  case $metric in l2) D=__USE_L2_DIST;; ip) D=__USE_IP_DIST;; cos) D=__USE_COS_DIST;; esac
  # main.cu:1-8 includes the C and C++ headers data.h relies on before it
  printf '#include <cstdio>\n#include <cstring>\n#include <string>\n#include <memory>\n#include "astar_accelerator.h"\n#include "warp_astar_accelerator.h"\n' > "$dir/unit.cu"
  "$NVCC" -cubin -gencode arch=compute_100,code=sm_100 -O3 -std=c++11 -w \
    -D$D -D__ENABLE_FIXHASH -D__ENABLE_VISITED_DEL -I"$dir" "$dir/unit.cu" \
    -o "$OUT/warp_astar_${metric}_d${dim}_pq${pq}_${measure}.cubin"
}
pids=()
for c in $CASES; do
  IFS=: read -r m d p <<< "$c"
  for meas in measure nomeasure; do
    build_one "$m" "$d" "$p" "$meas" &
    pids+=($!)
    if [ ${#pids[@]} -ge 8 ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
  done
done
wait
ls "$OUT"/*.cubin | wc -l
