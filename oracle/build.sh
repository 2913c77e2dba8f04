#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_build"
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    -o "$HERE/_build/libcochlea_oracle.so" "$HERE/cochlea_oracle.cpp" "$HERE/warmstart_oracle.cpp"
