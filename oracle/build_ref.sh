#!/usr/bin/env bash
# Builds, from the reference's own projector kernels
# (source/modules/reconstruction/Projector.cu, lines 22-785: the device and
# global functions, no host code):
#   oracle/_ref/libkvref.so          compiled for the CPU through ref_shim.h
#   oracle/_ref/ref_kernels.cubin    compiled for sm_103a as the reference
#                                    ships them (nvcc defaults, FMA contraction on)
#   oracle/_ref/ref_kernels_nofma.cubin  the same with -fmad=false
# (the cubins only when nvcc is on PATH), and from the reference's geometry
# module (source/modules/geometry/*.cpp with the vendored
# source/commons/tinyXML/tinyxml2.cpp, compiled where they lie):
#   oracle/_ref/ref_geometry         the reference's XML geometry reader behind
#                                    ref_geometry_driver.cpp; two headers that
#                                    gcc rejects are replaced by the stand-ins
#                                    in ref_geometry_shim/ (first on the
#                                    include path); TomoGeometryErrorCode.cpp is
#                                    left out (unused by the reader)
#   oracle/_ref/ref_drivers          the reference's ART and MLEM drivers
#                                    (Reconstructors.h) with PhantomMaker's
#                                    uniform start, behind ref_drivers_main.cpp,
#                                    on the host build of the reference kernels
#                                    (libkvref.so) through the Projector
#                                    stand-in in ref_driver_shim/ and the VTK
#                                    stand-ins in ref_vtk_stub/ (those of the
#                                    shift-and-add filters compute nothing and
#                                    record the shift rule's rows)
#   oracle/_ref/ref_histogram        the reference's histogram tools
#                                    (source/commons/HistogramMatchingTools.h)
#                                    behind ref_histogram_driver.cpp, against
#                                    the VTK stand-ins in ref_vtk_stub/ (the
#                                    header needs only an unsigned-short image)
# TEST INFRASTRUCTURE: checkers for the RC restatement in kvtomo_oracle.c and
# for the engine's RC kernels, the "reference GPU" timing line, and the
# checker for the drop-in's XML geometry reader.
#
# Usage: oracle/build_ref.sh <reference-root>   (oracle/build.py passes it)
# The kernel lines are extracted into oracle/_ref/ only for the compile and
# removed afterwards; only the shared library stays.  Exits 0 without building
# when the reference tree is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
if [ $# -lt 1 ]; then
    echo "usage: $0 <reference-root>" >&2
    exit 2
fi
ref="$1"
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
if command -v nvcc > /dev/null; then
    sed -n '22,785p' "$src" > "$out/ref_kernels_gpu.inc"
    nvcc -std=c++17 -O3 -cubin -gencode arch=compute_103a,code=sm_103a -w \
        -I "$out" "$here/ref_gpu_wrap.cu" -o "$out/ref_kernels.cubin" &
    nvcc -std=c++17 -O3 -cubin -gencode arch=compute_103a,code=sm_103a -w -fmad=false \
        -I "$out" "$here/ref_gpu_wrap.cu" -o "$out/ref_kernels_nofma.cubin" &
    wait
    rm -f "$out/ref_kernels_gpu.inc"
    echo "build_ref: built $out/ref_kernels.cubin, $out/ref_kernels_nofma.cubin"
fi
# the reference's geometry module, tinyxml2, PhantomMaker and the error
# categories, compiled once (in parallel) for the two checkers below
flags=(-std=c++17 -O1 -w -fpermissive -include cstring -include climits -I "$here/ref_driver_shim"
       -I "$here/ref_geometry_shim" -I "$here/ref_vtk_stub" -I "$ref/source")
obj="$out/obj"
mkdir -p "$obj"
geo=()
for f in "$ref"/source/modules/geometry/*.cpp "$ref/source/commons/tinyXML/tinyxml2.cpp"; do
    case "$f" in *_test.cpp|*/TomoGeometryErrorCode.cpp) continue ;; esac
    geo+=("$f")
done
extra=("$ref/source/modules/dataHandling/PhantomMaker.cpp" "$ref/source/commons/TomoErrorCondition.cpp"
       "$ref/source/modules/reconstruction/ReconstructorsErrorCode.cpp")
pids=()
for f in "${geo[@]}" "${extra[@]}"; do
    g++ "${flags[@]}" -c "$f" -o "$obj/$(basename "$f" .cpp).o" &
    pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
geo_obj=()
for f in "${geo[@]}"; do geo_obj+=("$obj/$(basename "$f" .cpp).o"); done
g++ "${flags[@]}" "$here/ref_geometry_driver.cpp" "${geo_obj[@]}" -o "$out/ref_geometry"
echo "build_ref: built $out/ref_geometry"
g++ "${flags[@]}" "$here/ref_drivers_main.cpp" "$obj"/*.o -L "$out" -lkvref -fopenmp \
    -Wl,-rpath,'$ORIGIN' -o "$out/ref_drivers"
rm -rf "$obj"
echo "build_ref: built $out/ref_drivers"
g++ -std=c++17 -O1 -w -fpermissive -include climits -I "$here/ref_vtk_stub" -I "$ref/source" \
    "$here/ref_histogram_driver.cpp" -o "$out/ref_histogram"
echo "build_ref: built $out/ref_histogram"
