#!/bin/sh
# Builds the reference's CUDA kernels, unmodified, from the reference's own
# source files into oracle/_ref/ (git-ignored). TEST/BASELINE INFRASTRUCTURE.
#
#   src/aggregation.cu (+ src/aggregation_kernels.cuh) -> _ref/ref_aggregation.cubin
#   src/breakage.cu    (+ src/breakage_kernels.cuh)    -> _ref/ref_breakage.cubin
#   examples/*/main.cpp, examples/common/pbe_examples_utils.hpp
#                                                      -> _ref/examples/ (staged as is)
#
# The six example programs are staged unchanged, beside the cubins, because
# the machine that runs the GPU tests has no reference checkout: the tests
# there compile them against this library's C++ headers (include/pbe_cuda)
# and link them twice, to libpbe_gb300.so and to the reference's own kernels
# (oracle/ref_dropin_shim.cpp), and compare what they print. oracle/_ref/ is
# git-ignored: nothing of the reference enters the repository's history.
#
# Only device code is built (nvcc -cubin), for sm_103a, with the reference's
# Release flags (-O3 -DNDEBUG, C++17). The reference's CMake forces an extra
# compute_86 target and needs cmake; it is not used. The host launch logic of
# src/aggregation.cu:16-61 and src/breakage.cu:14-79 is restated in
# oracle/ref_runner.cpp, which loads these cubins through the driver API.
# The cubins are CPU-architecture independent, so a copy built here runs on
# the aarch64 GPU machine as well.
set -e
# PBE_REFERENCE_DIR: the read-only reference checkout; /root/reference is
# where the build container mounts it.
REF="${PBE_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/aggregation.cu" ]; then
  echo "build_ref.sh: reference sources not found under $REF; keeping existing $OUT" >&2
  exit 0
fi
mkdir -p "$OUT"
# stage the example programs (plain copies; refreshed when the reference changes)
EXAMPLES="aggregation_constant aggregation_product aggregation_sum breakage_linear_symmetricbinary breakage_linear_uniform flocculation_two_stage"
mkdir -p "$OUT/examples/common"
if [ -f "$REF/examples/common/pbe_examples_utils.hpp" ]; then
  cp -p "$REF/examples/common/pbe_examples_utils.hpp" "$OUT/examples/common/"
  for ex in $EXAMPLES; do
    if [ -f "$REF/examples/$ex/main.cpp" ]; then
      mkdir -p "$OUT/examples/$ex"
      cp -p "$REF/examples/$ex/main.cpp" "$OUT/examples/$ex/main.cpp"
    fi
  done
fi
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
