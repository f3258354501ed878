#!/usr/bin/env bash
# Builds oracle/_ref/librayt_ref.so: the reference's own host pipeline
# (renderer, feedback extractor, GPU sort/scan, block cache, loader, builder,
# camera) and its OpenCL kernels compiled as C++, linked against the fake
# OpenCL runtime in oracle/ref_harness/.  Only the development container has
# the reference sources; outputs go to oracle/_ref/ only.
#
# The .cl kernels are copied into oracle/_ref/cl/ with one mechanical rewrite:
# OpenCL vector literals "(float4)(a, b, c, d)" become "float4(a, b, c, d)".
#
#   RAYT_REFERENCE=<reference checkout> bash oracle/build_ref.sh
set -euo pipefail
[ -n "${RAYT_REFERENCE:-}" ] || { echo "set RAYT_REFERENCE to the reference checkout (the directory holding rayt/)" >&2; exit 3; }
REF="$RAYT_REFERENCE/rayt"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
[ -d "$REF" ] || { echo "reference sources not found at $REF" >&2; exit 3; }
mkdir -p "$OUT/cl" "$OUT/obj"

for f in "$REF/GPU_renderer/kernels/"*.cl "$REF/GPU algorithms/kernels/"*.cl; do
  sed -E 's/\((float4|uchar4|uint2|char4)\)\(/\1(/g' "$f" > "$OUT/cl/$(basename "$f")"
done

CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O2 -fPIC -fopenmp -ffp-contract=off -fno-strict-aliasing -w
       -I "$HERE/ref_harness/shim" -I "$HERE/ref_harness" -I "$OUT/cl"
       -I "$REF/util" -I "$REF/CPU data" -I "$REF/GPU data" -I "$REF/GPU algorithms"
       -I "$REF/GPU_renderer" -I "$REF/scene" -I "$REF/scene sources")

SRC=(
  "$REF/util/buffer.cpp" "$REF/util/binary-util.cpp" "$REF/util/binary-file.cpp"
  "$REF/util/mat.cpp" "$REF/util/intersections.cpp"
  "$REF/CPU data/octree-constants.cpp" "$REF/CPU data/stored-octree-channel.cpp"
  "$REF/CPU data/stored-octree-channel-set.cpp" "$REF/CPU data/stored-octree-header.cpp"
  "$REF/CPU data/stored-octree-loader.cpp" "$REF/CPU data/stored-octree-raw-writer.cpp"
  "$REF/CPU data/stored-octree-traverser.cpp" "$REF/CPU data/stored-octree-writer.cpp"
  "$REF/GPU data/gpu-octree-channel.cpp" "$REF/GPU data/gpu-octree-data.cpp"
  "$REF/GPU data/gpu-octree-cache.cpp" "$REF/GPU data/gpu-octree-cache-manager.cpp"
  "$REF/GPU algorithms/gpu-sort.cpp" "$REF/GPU algorithms/gpu-scan.cpp"
  "$REF/GPU_renderer/gpu-ray-tracer.cpp" "$REF/GPU_renderer/ray-tracing-feedback-extractor.cpp"
  "$REF/scene/camera.cpp" "$REF/scene sources/stored-octree-test.cpp"
  "$HERE/ref_harness/fake_cl.cpp" "$HERE/ref_harness/stopwatch_linux.cpp"
  "$HERE/ref_harness/cl_init.cpp" "$HERE/ref_harness/cl_pass.cpp" "$HERE/ref_harness/cl_finish.cpp"
  "$HERE/ref_harness/cl_feedback.cpp" "$HERE/ref_harness/cl_sort_scan.cpp" "$HERE/ref_harness/cl_depth.cpp"
  "$HERE/ref_harness/ref_api.cpp"
)

pids=()
objs=()
i=0
for s in "${SRC[@]}"; do
  o="$OUT/obj/$i-$(basename "${s%.cpp}" | tr ' ' '_').o"
  objs+=("$o")
  "$CXX" "${FLAGS[@]}" -c "$s" -o "$o" &
  pids+=($!)
  i=$((i + 1))
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -shared -fopenmp -o "$OUT/librayt_ref.so" "${objs[@]}"
echo "built $OUT/librayt_ref.so"
