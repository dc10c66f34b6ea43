#!/bin/sh
# Builds oracle/_ref/libref.so: the reference's own runtime sources, compiled
# unmodified from where they lie, plus oracle/ref_shim.cpp (flat C entry points
# used by the parity tests). Only the six crypto sources are taken; myfpga.cpp,
# test.cpp and apps/*.cpp need the AWS FPGA SDK and are left out.
#
# This recipe is the one place that locates the reference checkout: the first
# argument, else $FHEACC_REFERENCE_ROOT, else /root/reference. It leaves a
# link oracle/_ref/reference to that checkout, through which the tests and the
# fixture scripts read the reference's headers and transcripts; where the
# reference is not mounted (exit 3) neither the library nor the link exists.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
set -e
REF="${1:-${FHEACC_REFERENCE_ROOT:-/root/reference}}"
SRC="$REF/FHE_ACC_runtime/src"
INC="$REF/FHE_ACC_runtime/include"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$SRC/RLWE.cpp" ]; then
    echo "reference sources not found under $REF; oracle/_ref not built" >&2
    exit 3
fi
mkdir -p "$OUT"
ln -sfn "$REF" "$OUT/reference"
if [ -f "$OUT/libref.so" ] && [ "$OUT/libref.so" -nt "$HERE/ref_shim.cpp" ]; then
    echo "up to date: $OUT/libref.so"
    exit 0
fi
g++ -std=c++14 -O3 -fPIC -shared -w -I"$INC" \
    "$SRC/nbt.cpp" "$SRC/params.cpp" "$SRC/RNG.cpp" "$SRC/LWE.cpp" "$SRC/RLWE.cpp" "$SRC/app.cpp" \
    "$HERE/ref_shim.cpp" -o "$OUT/libref.so.tmp"
mv "$OUT/libref.so.tmp" "$OUT/libref.so"
echo "built $OUT/libref.so"
