#!/bin/sh
# Host-compiler wrapper for the reference cubin build (passed to nvcc as the
# host compiler through a directory holding gcc/g++ links to this script).
# After a preprocessing step it deletes the reference's "#pragma message"
# lines: one of them prints __CUDA_ARCH__, which expands to a number the CUDA
# front end rejects inside that pragma (include/cochlea.cuh:69).  They are
# diagnostics only; every other line is passed through unchanged.
real="${REF_HOST_CC:-g++}"
out=""
pre=0
prev=""
for a in "$@"; do
  [ "$a" = "-E" ] && pre=1
  [ "$prev" = "-o" ] && out="$a"
  prev="$a"
done
"$real" "$@" || exit $?
if [ "$pre" = 1 ] && [ -n "$out" ] && [ -f "$out" ]; then
  sed -i '/^[[:space:]]*#pragma message/d' "$out"
fi
