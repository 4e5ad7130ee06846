#!/bin/sh
# Write tests/golden/refcuda_grid{4,8}.bin and refstructured_grid{4,8}.bin: final
# states of the reference's own CUDA kernels run on a GB300 -- the plain
# gridwide-independent kernels and the structured (gridwide-structured-cta32)
# kernel.  Two halves:
#  1. where the reference tree is present:
#       WITH_CUBIN=1 WITH_STRUCTURED=1 sh oracle/build_ref.sh
#     (builds oracle/_ref/ref_kernels.cubin and ref_structured.cubin from
#     reproducer.cpp, the latter with the slice headers that the reference's own
#     tools/slice_dag.py generates)
#  2. on the GPU machine, from the repository root:
#       sh tests/golden/make_refcuda_fixtures.sh <outdir>
#     then copy <outdir>/ref*_grid*.bin into tests/golden/.
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
    if [ -f oracle/_ref/ref_structured.cubin ]; then
        "$OUT/ref_cuda_launcher" oracle/_ref/ref_structured.cubin $g "$OUT/refstructured_grid$g.bin" --structured
    fi
done
