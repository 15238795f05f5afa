#!/bin/sh
# Builds the reference's CUDA kernels, unmodified, from the reference's own
# source files into oracle/_ref/ (git-ignored). TEST/BASELINE INFRASTRUCTURE.
#
#   src/aggregation.cu (+ src/aggregation_kernels.cuh) -> _ref/ref_aggregation.cubin
#   src/breakage.cu    (+ src/breakage_kernels.cuh)    -> _ref/ref_breakage.cubin
#
# Only device code is built (nvcc -cubin), for sm_103a, with the reference's
# Release flags (-O3 -DNDEBUG, C++17). The reference's CMake forces an extra
# compute_86 target and needs cmake; it is not used. The host launch logic of
# src/aggregation.cu:16-61 and src/breakage.cu:14-79 is restated in
# oracle/ref_runner.cpp, which loads these cubins through the driver API.
# The cubins are CPU-architecture independent, so a copy built here runs on
# the aarch64 GPU machine as well.
set -e
REF="${PBE_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/aggregation.cu" ]; then
  echo "build_ref.sh: reference sources not found under $REF; keeping existing $OUT" >&2
  exit 0
fi
mkdir -p "$OUT"
up_to_date=1
for pair in "aggregation:aggregation_kernels" "breakage:breakage_kernels"; do
  name=${pair%%:*}; hdr=${pair##*:}
  cub="$OUT/ref_$name.cubin"
  if [ ! -f "$cub" ] || [ "$REF/src/$name.cu" -nt "$cub" ] || [ "$REF/src/$hdr.cuh" -nt "$cub" ]; then up_to_date=0; fi
done
if [ "$up_to_date" = 1 ] && [ "${1:-}" != "--force" ]; then exit 0; fi
NVCC="${NVCC:-nvcc}"
FLAGS="-cubin -gencode arch=compute_103a,code=sm_103a -O3 -DNDEBUG -std=c++17 -I$REF/include -I$REF/src"
$NVCC $FLAGS "$REF/src/aggregation.cu" -o "$OUT/ref_aggregation.cubin" &
P1=$!
$NVCC $FLAGS "$REF/src/breakage.cu" -o "$OUT/ref_breakage.cubin" &
P2=$!
wait $P1
wait $P2
echo "built $OUT/ref_aggregation.cubin $OUT/ref_breakage.cubin"
