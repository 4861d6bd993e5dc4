#!/bin/bash
# Builds the reference's own code from its sources under the reference tree into
# oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE ONLY; needs the reference tree, so it
# runs where that tree is mounted (not on the GPU host).
#   mf-train, mf-predict   test/{mf.cpp,mf-train.cpp,mf-predict.cpp}, flags of test/Makefile
#   ref_rmse               calc_rmse/mf_load_model/read_problem from test/mf.cpp
#   ref_layout             singleGPU/sgd.cu host functions (id maps, shuffle, grid, scale)
#   transform              data/netflix/transform.cpp (rating text -> 12-byte records)
set -euo pipefail
REF=${CUMF_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
mkdir -p "$OUT"
[ -d "$REF/test" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
DFLAG="-DUSEOMP"
case "$(uname -m)" in x86_64) DFLAG="$DFLAG -DUSESSE"; MARCH="-march=native";; *) MARCH="";; esac
CXXFLAGS="-Wall -O3 -pthread -std=c++0x $MARCH -fopenmp -w"
g++ $CXXFLAGS $DFLAG -c -fPIC -o "$OUT/mf.o" "$REF/test/mf.cpp"
g++ $CXXFLAGS $DFLAG -o "$OUT/mf-train" "$REF/test/mf-train.cpp" "$OUT/mf.o"
g++ $CXXFLAGS $DFLAG -o "$OUT/mf-predict" "$REF/test/mf-predict.cpp" "$OUT/mf.o"
g++ $CXXFLAGS $DFLAG -I"$REF/test" -o "$OUT/ref_rmse" "$HERE/ref_rmse_driver.cpp" "$OUT/mf.o"
# sgd.cu compiled as the reference ships it (host part for this machine, device part for sm_103a).
nvcc -std=c++11 -O3 -w -gencode arch=compute_103a,code=sm_103a -I"$REF/singleGPU" \
     -c "$REF/singleGPU/sgd.cu" -o "$OUT/sgd.o"
nvcc -std=c++11 -O3 -w -Wno-deprecated-declarations -I"$REF/singleGPU" \
     -c "$HERE/ref_layout_driver.cpp" -o "$OUT/ref_layout_driver.o"
nvcc -o "$OUT/ref_layout" "$OUT/ref_layout_driver.o" "$OUT/sgd.o" -Xlinker --wrap=time -lcurand
g++ -O2 -w -o "$OUT/transform" "$REF/data/netflix/transform.cpp"
echo "built reference tools in $OUT"
