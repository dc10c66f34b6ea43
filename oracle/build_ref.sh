#!/bin/sh
# Builds oracle/_ref/libref.so: the reference's own runtime sources, compiled
# unmodified from where they lie, plus oracle/ref_shim.cpp (flat C entry points
# used by the parity tests). Only the six crypto sources are taken; myfpga.cpp,
# test.cpp and apps/*.cpp need the AWS FPGA SDK and are left out.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -e
REF="${1:-/root/reference}"
SRC="$REF/FHE_ACC_runtime/src"
INC="$REF/FHE_ACC_runtime/include"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$SRC/RLWE.cpp" ]; then
    echo "reference sources not found under $REF; oracle/_ref not built" >&2
    exit 3
fi
mkdir -p "$OUT"
g++ -std=c++14 -O3 -fPIC -shared -w -I"$INC" \
    "$SRC/nbt.cpp" "$SRC/params.cpp" "$SRC/RNG.cpp" "$SRC/LWE.cpp" "$SRC/RLWE.cpp" "$SRC/app.cpp" \
    "$HERE/ref_shim.cpp" -o "$OUT/libref.so.tmp"
mv "$OUT/libref.so.tmp" "$OUT/libref.so"
echo "built $OUT/libref.so"
