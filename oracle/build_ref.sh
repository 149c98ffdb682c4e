#!/bin/sh
# Builds test oracles from the reference's own sources, where they lie, into
# oracle/_ref/ (git-ignored).  Test and measurement infrastructure only; run in
# the container that has the reference checkout.
#
#   ref_loader             the reference's dataset loader (dataset.cu, host C++)
#   ref_<variant>.cubin    the reference's join kernels (kernel_join.cu) for
#                          sm_103a, one cubin per compile-time configuration
#                          (params.h: INPUT_DATA_DIM, COMPUTE_DIM,
#                          COMPUTE_PREC, ACCUM_PREC); run on the GPU by
#                          oracle/ref_gpu.cu, which loads them with the driver
#                          API and launches them as gpu_join.cu:210-322 does
#
# The reference sets its configuration in params.h (params.h:4-12), so each
# variant compiles a transient copy of kernel_join.cu / kernel_join.h with an
# edited params.h under oracle/_ref/src_<variant>/, deleted right after.  The
# FP64 variants also wrap the two FP16-only kernels (TensorBasic and
# TensorHalf, kernel_join.cu:244-524), which do not compile with double
# fragments, in `#if COMPUTE_PREC != 64` -- the guard the reference's own
# gpu_join.cu:296 would need as well.  Nothing else is changed.  The
# "nofma" variant is the FP64 one compiled with -fmad=false (no contraction),
# to show what the other reading of kernel_join.cu:186-189 would count.
#
# Usage: oracle/build_ref.sh <reference-root>
set -e
[ $# -ge 1 ] || { echo "usage: $0 <reference-root>" >&2; exit 2; }
REF="$1"
HERE="$(cd "$(dirname "$0")" && pwd)"
[ -f "$REF/dataset.cu" ] || { echo "reference not found at $REF" >&2; exit 1; }
OUT="$HERE/_ref"
mkdir -p "$OUT"
g++ -O2 -std=c++14 -I"$REF" -x c++ "$REF/dataset.cu" -x none "$HERE/ref_loader_main.cpp" \
    -o "$OUT/ref_loader"
echo "built $OUT/ref_loader"

NVCC="${NVCC:-nvcc}"
command -v "$NVCC" >/dev/null 2>&1 || { echo "nvcc not found: reference kernels not built"; exit 0; }

# variant <name> <INPUT_DATA_DIM> <COMPUTE_DIM> <COMPUTE_PREC> <ACCUM_PREC> [nvcc flags]
variant() {
    name=$1; din=$2; dcomp=$3; cprec=$4; aprec=$5; shift 5
    src="$OUT/src_$name"
    rm -rf "$src"
    mkdir -p "$src"
    cp "$REF/kernel_join.cu" "$REF/kernel_join.h" "$src/"
    sed -e "s/^#define INPUT_DATA_DIM .*/#define INPUT_DATA_DIM $din/" \
        -e "s/^#define COMPUTE_DIM .*/#define COMPUTE_DIM $dcomp/" \
        -e "s/^#define COMPUTE_PREC .*/#define COMPUTE_PREC $cprec/" \
        -e "s/^#define ACCUM_PREC .*/#define ACCUM_PREC $aprec/" \
        "$REF/params.h" > "$src/params.h"
    if [ "$cprec" = 64 ]; then
        sed -i -e '/^__global__ void distanceCalculationBruteForceTensorBasic(/i #if COMPUTE_PREC != 64' \
               -e '/^#if COMPUTE_PREC == 64/i #endif' "$src/kernel_join.cu"
    fi
    # the reference's makefile flags (makefile:6), C++17 for CUDA 13's headers
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -lineinfo -w "$@" \
        -I"$src" "$src/kernel_join.cu" -o "$OUT/ref_$name.cubin"
    rm -rf "$src"
    echo "built $OUT/ref_$name.cubin"
}

# FP16 MQ path as shipped (INPUT 64 / COMPUTE 16 / ACCUM 32) at the benchmark dims
variant fp16_d64 64 64 16 32
variant fp16_d128 128 128 16 32
# FP64 (INPUT 64 / COMPUTE 64 / ACCUM 64): TensorDouble and the CUDA-core kernel
variant fp64_d64 64 64 64 64
variant fp64_d128 128 128 64 64
# FP64 CUDA-core kernel at the golden fixtures' dims (d = 18 and 3)
variant fp64_d18 18 20 64 64
variant fp64_d3 3 4 64 64
variant fp64_d18_nofma 18 20 64 64 -fmad=false
