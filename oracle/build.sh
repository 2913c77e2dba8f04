#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/, and the
# launcher of the reference's own kernels (oracle/ref_gpu.cpp, driver API).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_build"
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    -o "$HERE/_build/libcochlea_oracle.so" "$HERE/cochlea_oracle.cpp" "$HERE/warmstart_oracle.cpp"
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
g++ -std=c++17 -O2 -fPIC -shared -I "$CUDA_HOME/include" \
    -o "$HERE/_build/libref_gpu.so" "$HERE/ref_gpu.cpp" \
    -L "$CUDA_HOME/lib64/stubs" -L "$CUDA_HOME/lib64" -lcuda
