#!/usr/bin/env bash
# Stage the reference's sources of the hot path (src/, inst/cuda/) into
# baseline/_ref/gputools, which git ignores and the GPU hosts receive with
# the working tree, so that the reference's own CPU loops and GPU path can be
# built and run there (oracle/build_ref.sh, oracle/build_ref_gpu.sh) where the
# reference tree itself is absent.  Test infrastructure only.
# Usage: stage_ref.sh <reference tree>
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$HERE")"
REF=${1:?usage: stage_ref.sh <reference tree>}
DST="$ROOT/baseline/_ref/gputools"
if [ ! -f "$REF/src/correlation.cpp" ]; then
  echo "no reference tree at $REF" >&2
  exit 1
fi
mkdir -p "$DST/src" "$DST/inst/cuda"
cp "$REF"/src/*.cpp "$REF"/src/*.h "$DST/src/"
cp "$REF"/inst/cuda/*.cu "$DST/inst/cuda/"
echo "staged $REF into $DST"
