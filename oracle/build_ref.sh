#!/bin/sh
# Builds the reference's own dataset loader (dataset.cu, plain host C++) from
# the reference sources where they lie, into oracle/_ref/.  Test
# infrastructure only; run in the container that has the reference mounted.
# Usage: oracle/build_ref.sh <reference-root>
set -e
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
[ -f "$REF/dataset.cu" ] || { echo "reference not found at $REF" >&2; exit 1; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++14 -I"$REF" -x c++ "$REF/dataset.cu" -x none "$HERE/ref_loader_main.cpp" \
    -o "$HERE/_ref/ref_loader"
echo "built $HERE/_ref/ref_loader"
