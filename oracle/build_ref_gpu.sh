#!/usr/bin/env bash
# Build the reference's own GPU path (host orchestration in src/*.cpp and
# kernels in inst/cuda/*.cu, from a staged copy of the reference tree) into
# baseline/_ref/libref_gpu.so, for tests/golden/make_golden_gpu.py to record
# what the reference returns.  Test infrastructure: the library is never
# shipped and nothing in gputools_gb300 links it.
#
# The kernels are compiled by nvcc for sm_103a with --use_fast_math, the one
# option the reference gives NVRTC (src/cudaUtils.cpp:144); they are launched
# by name through oracle/ref_shim/gpu_shim.cpp instead of a per-launch NVRTC
# module load.  Usage: build_ref_gpu.sh [staged tree, default
# baseline/_ref/gputools].
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$HERE")"
REF=${1:-$ROOT/baseline/_ref/gputools}
OUT="$ROOT/baseline/_ref"
CUDA=${CUDA_HOME:-/usr/local/cuda}
NVCC="$CUDA/bin/nvcc"
if [ ! -f "$REF/src/correlation.cpp" ] || [ ! -f "$REF/inst/cuda/correlation.cu" ]; then
  echo "staged reference tree not found at $REF; skipping libref_gpu.so" >&2
  exit 0
fi
if [ ! -x "$NVCC" ]; then
  echo "nvcc not found; skipping libref_gpu.so" >&2
  exit 0
fi
OBJ="$OUT/_obj_gpu"
mkdir -p "$OBJ"
ARCH="-gencode arch=compute_103a,code=sm_103a"
pids=()
for k in correlation distance kendall mi hcluster; do
  extra=""
  [ "$k" = hcluster ] && extra="-include math_constants.h"
  "$NVCC" $ARCH -O3 --use_fast_math -w -std=c++17 -Xcompiler -fPIC $extra \
    -I"$REF/inst/cuda" -I"$HERE/ref_shim" \
    -c "$HERE/ref_shim/ref_kernels_$k.cu" -o "$OBJ/ref_kernels_$k.o" &
  pids+=($!)
done
for f in correlation distance kendall mi hcluster; do
  g++ -O3 -fPIC -std=c++17 -w -include "$HERE/ref_shim/compat.h" \
    -I"$HERE/ref_shim" -I"$REF/src" -I"$CUDA/include" \
    -c "$REF/src/$f.cpp" -o "$OBJ/host_$f.o" &
  pids+=($!)
done
g++ -O3 -fPIC -std=c++17 -w -I"$HERE/ref_shim" -I"$REF/src" -I"$CUDA/include" \
  -c "$HERE/ref_shim/gpu_shim.cpp" -o "$OBJ/gpu_shim.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" $ARCH -shared -o "$OUT/libref_gpu.so" "$OBJ"/*.o -lcublas -ldl -lpthread -lrt
echo "built $OUT/libref_gpu.so"
