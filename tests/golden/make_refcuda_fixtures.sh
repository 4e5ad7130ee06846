#!/bin/sh
# Write tests/golden/refcuda_grid{4,8}.bin: final states of the reference's own
# CUDA kernels run on a GB300.  Two halves:
#  1. where the reference tree is present:  WITH_CUBIN=1 sh oracle/build_ref.sh
#     (builds oracle/_ref/ref_kernels.cubin from reproducer.cpp)
#  2. on the GPU machine, from the repository root:
#     sh tests/golden/make_refcuda_fixtures.sh <outdir>
#     then copy <outdir>/refcuda_grid*.bin into tests/golden/.
# Without <outdir> the files go to a fresh temporary directory (printed).
set -e
OUT=${1:-$(mktemp -d)}
echo "writing to $OUT"
mkdir -p "$OUT"
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
g++ -O2 -std=c++17 -I"$CUDA_HOME/include" -o "$OUT/ref_cuda_launcher" oracle/ref_cuda_launcher.cpp \
    -L"$CUDA_HOME/lib64/stubs" -L"$CUDA_HOME/targets/sbsa-linux/lib/stubs" -lcuda
for g in 4 8; do
    "$OUT/ref_cuda_launcher" oracle/_ref/ref_kernels.cubin $g "$OUT/refcuda_grid$g.bin"
done
