#!/usr/bin/env bash
# Compile the reference's own host code for the TC preprocessing / two-hop counting and
# the SI data generator, unmodified, from the sources where they lie under the reference
# checkout, into oracle/_ref/ref_driver. TEST INFRASTRUCTURE ONLY: used to generate the
# golden vectors under tests/golden/ that pin the oracle.
#
#   REF=/path/to/RT-Graph oracle/build_ref.sh
#
# Without REF the checkout is looked up next to this repository (../reference).
#
# Reference files used (read-only): tc/graph/graph.cpp, tc/bs_tc/bs_tc.cu (its host
# function Preprocessing for the driver; its method-0 kernel ListIntersectionKernel as a
# cubin for the benchmark's reference GPU data point, oracle/ref_gpu.py),
# set_intersection/data_generator/data.cpp. ThrustSortEdgesInBatch is provided on the
# host by oracle/ref_shim.cpp. CCCL 3 no longer pulls <vector>, <algorithm> and <cassert>
# into bs_tc.cu, so they are force-included.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-$HERE/../../reference}"
OUT="$HERE/_ref"
CUDA_HOME="${CUDA_HOME:-/usr/local/cuda}"
if [ ! -d "$REF/tc/graph" ]; then
  echo "reference sources not found at $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
INC="-I$REF/tc/graph/include -I$REF/tc/utils -I$REF/tc/bs_tc -I$REF/set_intersection/data_generator -I$CUDA_HOME/include"
g++ -O2 -fopenmp -std=c++17 $INC -c "$REF/tc/graph/graph.cpp" -o "$OUT/graph.o" &
g++ -O2 -std=c++17 $INC -c "$REF/set_intersection/data_generator/data.cpp" -o "$OUT/data.o" &
nvcc -O2 -std=c++17 -Xcompiler -fopenmp -include vector -include algorithm -include cassert \
  $INC -gencode arch=compute_103a,code=sm_103a -c "$REF/tc/bs_tc/bs_tc.cu" -o "$OUT/bs_tc.o" &
g++ -O2 -std=c++17 $INC -c "$HERE/ref_shim.cpp" -o "$OUT/ref_shim.o" &
g++ -O2 -std=c++17 $INC -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" &
# the reference's own GPU triangle count, method 0 (ListIntersectionKernel), device code
# only: loaded and launched by oracle/ref_gpu.py through the CUDA driver API
nvcc -O3 -std=c++17 -cubin -gencode arch=compute_103a,code=sm_103a -include "$HERE/ref_method0.h" \
  -include vector -include algorithm -include cassert $INC -I"$REF/tc/rt_tc/include" \
  "$REF/tc/bs_tc/bs_tc.cu" -o "$OUT/bs_tc_method0.cubin" &
wait
g++ -fopenmp -o "$OUT/ref_driver" "$OUT/ref_driver.o" "$OUT/ref_shim.o" "$OUT/graph.o" \
  "$OUT/bs_tc.o" "$OUT/data.o" -L"$CUDA_HOME/lib64" -lcudart
echo "built $OUT/ref_driver"
