#!/bin/sh
# Builds oracle/_ref/cochlea_ref.cubin: the REFERENCE's own device code
# (src/cochlea.cu, which includes include/cochlea.cuh), compiled unmodified
# for sm_103a from the reference tree with the reference's default nvcc
# settings.  Test infrastructure only: it is the parity reference loaded by
# oracle/ref_gpu.cpp; the product never loads it.
#
# The reference is written for MSVC and the CUDA Samples; oracle/ref_shim/
# supplies stand-ins for helper_cuda.h, helper_functions.h and
# Boost.Stacktrace (used only by host code), a forced include that defines
# away `throw(...)` and memcpy_s, and a host-compiler wrapper that drops the
# diagnostic "#pragma message" lines from the preprocessed source.  The cubin
# holds device code only, so it runs on any host CPU with an sm_103a GPU.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${COCHLEA_REFERENCE:-/root/reference}
[ -f "$REF/src/cochlea.cu" ] || { echo "reference tree not present; skipping"; exit 0; }
OUT="$HERE/_ref"
CC="$OUT/host_cc"
mkdir -p "$OUT" "$CC"
ln -sf "$HERE/ref_shim/host_cc.sh" "$CC/gcc"
ln -sf "$HERE/ref_shim/host_cc.sh" "$CC/g++"
nvcc -ccbin "$CC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -w \
    -include pre.h -I "$HERE/ref_shim" -I "$REF/include" \
    "$REF/src/cochlea.cu" -o "$OUT/cochlea_ref.cubin.tmp"
mv "$OUT/cochlea_ref.cubin.tmp" "$OUT/cochlea_ref.cubin"
