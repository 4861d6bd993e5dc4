#!/bin/bash
# Builds the reference's own code into oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE ONLY.
#
#   mf-train, mf-predict   LIBMF, test/{mf.cpp,mf-train.cpp,mf-predict.cpp}, flags of test/Makefile
#                          (-DUSESSE -msse3 only on x86_64; -march=native nowhere)
#   cumf_sgd_ref           the reference GPU trainer singleGPU/{main.cpp,sgd.cu,sgd_kernel.cu},
#                          built for sm_103a with oracle/ref_shfl_shim.h force-included (CUDA 13
#                          has no maskless __shfl/__shfl_down); no other change
#   ref_rmse               calc_rmse/mf_load_model/read_problem from test/mf.cpp
#   ref_layout             singleGPU/sgd.cu host functions (id maps, shuffle, grid, scale)
#   transform              data/netflix/transform.cpp (rating text -> 12-byte records)
#
# Where the reference tree is mounted, everything builds from the sources where they lie, and
# the files that the three trainer tools need are also copied into oracle/_ref/src/
# (git-ignored like the rest of oracle/_ref, never committed): the GPU host has no reference
# tree and is an aarch64 machine that cannot run what this x86 machine builds, so it compiles
# mf-train, mf-predict and cumf_sgd_ref from that copy (second branch below).
set -euo pipefail
REF=${CUMF_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
STAGE=$OUT/src
mkdir -p "$OUT"

DFLAG="-DUSEOMP"
SIMD=""
case "$(uname -m)" in x86_64) DFLAG="$DFLAG -DUSESSE"; SIMD="-msse3";; esac
CXXFLAGS="-Wall -O3 -pthread -std=c++0x -fopenmp -w $SIMD"
NVARCH="-gencode arch=compute_103a,code=sm_103a"

wait_all() {  # waits for every background job; fails if any failed
    local rc=0 pid
    for pid in "$@"; do wait "$pid" || rc=1; done
    return $rc
}

build_trainers() {  # $1: directory holding singleGPU/ and test/
    local S=$1 p1 p2 p3 p4
    g++ $CXXFLAGS $DFLAG -c -fPIC -o "$OUT/mf.o" "$S/test/mf.cpp" & p1=$!
    nvcc -std=c++11 -O3 -w $NVARCH -Xcompiler -fopenmp -DUSEOMP -I"$S/singleGPU" \
         -c "$S/singleGPU/main.cpp" -o "$OUT/ref_main.o" & p2=$!
    nvcc -std=c++11 -O3 -w $NVARCH -Xcompiler -fopenmp -DUSEOMP -include "$HERE/ref_shfl_shim.h" \
         -I"$S/singleGPU" -c "$S/singleGPU/sgd.cu" -o "$OUT/ref_sgd.o" & p3=$!
    nvcc -std=c++11 -O3 -w $NVARCH -Xcompiler -fopenmp -DUSEOMP -include "$HERE/ref_shfl_shim.h" \
         -I"$S/singleGPU" -c "$S/singleGPU/sgd_kernel.cu" -o "$OUT/ref_sgd_kernel.o" & p4=$!
    wait_all $p1 $p2 $p3 $p4
    g++ $CXXFLAGS $DFLAG -o "$OUT/mf-train" "$S/test/mf-train.cpp" "$OUT/mf.o" & p1=$!
    g++ $CXXFLAGS $DFLAG -o "$OUT/mf-predict" "$S/test/mf-predict.cpp" "$OUT/mf.o" & p2=$!
    nvcc $NVARCH -o "$OUT/cumf_sgd_ref" "$OUT/ref_main.o" "$OUT/ref_sgd.o" "$OUT/ref_sgd_kernel.o" \
         -Xcompiler -fopenmp -lcurand -lrt & p3=$!
    wait_all $p1 $p2 $p3
    local simd=scalar
    case "$DFLAG" in *USESSE*) simd=sse;; esac
    echo "mf-train simd=$simd arch=$(uname -m)" > "$OUT/BUILD_INFO"
}

if [ -d "$REF/test" ] && [ -d "$REF/singleGPU" ]; then
    build_trainers "$REF"
    g++ $CXXFLAGS $DFLAG -I"$REF/test" -o "$OUT/ref_rmse" "$HERE/ref_rmse_driver.cpp" "$OUT/mf.o"
    # sgd.cu compiled as the reference ships it (host part for this machine, device part for sm_103a).
    nvcc -std=c++11 -O3 -w $NVARCH -I"$REF/singleGPU" -c "$REF/singleGPU/sgd.cu" -o "$OUT/sgd.o"
    nvcc -std=c++11 -O3 -w -Wno-deprecated-declarations -I"$REF/singleGPU" \
         -c "$HERE/ref_layout_driver.cpp" -o "$OUT/ref_layout_driver.o"
    nvcc -o "$OUT/ref_layout" "$OUT/ref_layout_driver.o" "$OUT/sgd.o" -Xlinker --wrap=time -lcurand
    g++ -O2 -w -o "$OUT/transform" "$REF/data/netflix/transform.cpp"
    mkdir -p "$STAGE/singleGPU" "$STAGE/test"
    for f in main.cpp sgd.cu sgd.h sgd_kernel.cu sgd_kernel.h sgd_k128_kernel_hogwild_warp32.h; do
        install -m 0644 "$REF/singleGPU/$f" "$STAGE/singleGPU/$f"
    done
    for f in mf.cpp mf.h mf-train.cpp mf-predict.cpp; do install -m 0644 "$REF/test/$f" "$STAGE/test/$f"; done
    echo "built reference tools in $OUT (trainer sources staged in $STAGE for the GPU host)"
elif [ -f "$STAGE/singleGPU/sgd_kernel.cu" ] && [ -f "$STAGE/test/mf.cpp" ]; then
    build_trainers "$STAGE"
    echo "built mf-train, mf-predict and cumf_sgd_ref in $OUT from the staged reference sources"
else
    echo "reference tree not found at $REF and no staged sources in $STAGE" >&2
    exit 1
fi
