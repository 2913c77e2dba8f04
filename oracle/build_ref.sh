#!/bin/sh
# Builds oracle/_ref/libref_pins.so from the reference's own sources
# (include/const.h, src/tridiag.cpp under /root/reference) plus the shim
# oracle/ref_pins.cpp.  Test infrastructure: used only to pin the oracle.
# The reference names its header "CVector.h" in places; a one-line forwarding
# header in the build directory resolves that name.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${COCHLEA_REFERENCE:-/root/reference}
[ -d "$REF/src" ] || { echo "reference tree not present; skipping"; exit 0; }
OUT="$HERE/_ref"
mkdir -p "$OUT/shim"
echo '#include "cvector.h"' > "$OUT/shim/CVector.h"
g++ -std=c++17 -O2 -fPIC -shared -ffp-contract=off -include iterator \
    -I "$OUT/shim" -I "$REF/include" \
    "$HERE/ref_pins.cpp" "$REF/src/tridiag.cpp" -o "$OUT/libref_pins.so"
