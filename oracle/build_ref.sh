#!/bin/sh
# Build the reference itself from its own sources into oracle/_ref/ (test
# infrastructure; nothing here is committed or shipped).  Needs the reference tree:
# REF_DIR, by default the checkout named "reference" beside this repository; exits
# 0 without building (and says where it looked) when it is absent.
#   oracle/_ref/libwr_ref.so         reference TU + C shim (ref_shim.cpp), CPU
#   oracle/_ref/reproducer_cpu       the unmodified reference CPU program
#   oracle/_ref/ref_kernels.cubin    reference CUDA device code for sm_103a
#                                    (ref_cuda_shim.cu), only with WITH_CUBIN=1
#   oracle/_ref/ref_structured.cubin the reference's structured (cta32) CUDA kernel,
#                                    only with WITH_STRUCTURED=1: its generated
#                                    slice headers are first written by the
#                                    reference's own slicer (tools/slice_dag.py, pure
#                                    Python, from reproducer.mojo) into
#                                    oracle/_ref/generated/
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_DIR=${REF_DIR:-$(cd "$HERE/../.." && pwd)/reference}
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/reproducer.cpp" ]; then
    echo "reference tree not found at $REF_DIR; oracle/_ref not built"
    exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
# -ffp-contract=off keeps a*b+c unfused on every host (aarch64 GCC fuses by default)
$CXX -std=c++20 -O2 -ffp-contract=off -fopenmp -fPIC -shared \
    -DREFERENCE_TU="\"$REF_DIR/reproducer.cpp\"" \
    -o "$OUT/libwr_ref.so" "$HERE/ref_shim.cpp" &
P1=$!
$CXX -std=c++20 -O3 -ffp-contract=off -o "$OUT/reproducer_cpu" "$REF_DIR/reproducer.cpp" &
P2=$!
P3=
if [ "${WITH_CUBIN:-0}" = "1" ]; then
    nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -std=c++20 \
        --expt-relaxed-constexpr --fmad=false --maxrregcount=255 \
        -DREFERENCE_TU="\"$REF_DIR/reproducer.cpp\"" \
        -o "$OUT/ref_kernels.cubin" "$HERE/ref_cuda_shim.cu" &
    P3=$!
fi
P4=
if [ "${WITH_STRUCTURED:-0}" = "1" ]; then
    PYTHON=${PYTHON:-python3}
    $PYTHON -c "import sys; from pathlib import Path; sys.path.insert(0, sys.argv[1] + '/tools'); import slice_dag; slice_dag.generate(Path(sys.argv[1]) / 'reproducer.mojo', Path(sys.argv[2]))" "$REF_DIR" "$OUT/generated"
    nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -std=c++20 \
        --expt-relaxed-constexpr --fmad=false --maxrregcount=255 \
        -DPRIMORDIAL_ROS2S_CUDA_STRUCTURED -I "$OUT" \
        -DREFERENCE_TU="\"$REF_DIR/reproducer.cpp\"" \
        -o "$OUT/ref_structured.cubin" "$HERE/ref_cuda_shim.cu" &
    P4=$!
fi
wait $P1
wait $P2
[ -z "$P3" ] || wait $P3
[ -z "$P4" ] || wait $P4
echo "built $(ls "$OUT")"
