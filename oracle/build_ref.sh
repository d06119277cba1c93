#!/usr/bin/env bash
# Builds oracle/_ref/libkvref.so: the reference's own projector kernels
# (source/modules/reconstruction/Projector.cu, lines 22-785: the device and
# global functions, no host code) compiled for the CPU through ref_shim.h.
# TEST INFRASTRUCTURE: a checker for the RC restatement in kvtomo_oracle.c.
#
# Usage: oracle/build_ref.sh [reference-root]   (default /root/reference)
# The kernel lines are extracted into oracle/_ref/ only for the compile and
# removed afterwards; only the shared library stays.  Exits 0 without building
# when the reference tree is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-/root/reference}"
src="$ref/source/modules/reconstruction/Projector.cu"
out="$here/_ref"
if [ ! -f "$src" ]; then
    echo "build_ref: reference tree not found at $ref; skipping" >&2
    exit 0
fi
mkdir -p "$out"
sed -n '22,785p' "$src" > "$out/ref_kernels_cpu.inc"
g++ -std=c++17 -O2 -fPIC -shared -fopenmp -fpermissive -ffp-contract=off -w \
    -I "$here" -I "$out" "$here/ref_driver.cpp" -o "$out/libkvref.so"
rm -f "$out/ref_kernels_cpu.inc"
echo "build_ref: built $out/libkvref.so"
