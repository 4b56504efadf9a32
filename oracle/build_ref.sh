#!/usr/bin/env bash
# Compile the reference's own CPU loops (distance_host in src/distance.cpp,
# hostKendall / permHostKendall / hostSignif in src/correlation.cpp) straight
# from the read-only reference tree into oracle/_ref/libref_cpu.so.
# Only builds where the reference tree exists (not on the GPU hosts); the
# result is test infrastructure used to pin the oracle, never shipped.
# The tree's location comes from GPUTOOLS_REFERENCE (oracle.build() sets it
# from the benchmark's reference_path).
set -euo pipefail
REF=${GPUTOOLS_REFERENCE:-}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
CUDA=${CUDA_HOME:-/usr/local/cuda}
if [ -z "$REF" ] || [ ! -f "$REF/src/distance.cpp" ]; then
  echo "reference tree not found (GPUTOOLS_REFERENCE='$REF'); skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -O3 -fPIC -shared -std=c++17 -w \
  -include "$HERE/ref_shim/compat.h" \
  -I"$HERE/ref_shim" -I"$REF/src" -I"$CUDA/include" \
  "$REF/src/distance.cpp" "$REF/src/correlation.cpp" "$HERE/ref_shim/shim.cpp" \
  -L"$CUDA/lib64" -lcublas -lcudart_static -ldl -lpthread -lrt \
  -Wl,-rpath,"$CUDA/lib64" \
  -o "$OUT/libref_cpu.so"
echo "built $OUT/libref_cpu.so"
