#!/usr/bin/env bash
# Compile the reference's own CUDA sources, unmodified and where they lie, into
# device-only cubins for sm_103a under oracle/_ref/ (git-ignored).  The reference's CMake
# turns on separable compilation (CMakeLists.txt:56), so each unit is compiled with
# -rdc=true and then device-linked by nvlink into a loadable cubin.  The cubins carry no
# host code, so a copy built on an x86 host also runs on the Arm GPU host, where the
# reference sources are absent.  oracle/refkern.py launches them for golden vectors.
set -euo pipefail
SRC="${REF_SRC:-/root/reference/pystrns2cards/src}"
OUT="$(cd "$(dirname "$0")" && pwd)/_ref"
if [ ! -d "$SRC" ]; then
  echo "build_ref.sh: reference sources not found at $SRC; keeping existing cubins" >&2
  exit 0
fi
mkdir -p "$OUT"
pids=()
for u in dda rasterize antialias bitset_utils compact_utils curve_utils; do
  if [ ! -f "$OUT/$u.cubin" ] || [ "$SRC/$u.cu" -nt "$OUT/$u.cubin" ]; then
    ( nvcc -cubin -rdc=true -gencode arch=compute_103a,code=sm_103a -o "$OUT/$u.rdc.cubin" "$SRC/$u.cu" &&
      nvlink -arch=sm_103a -o "$OUT/$u.cubin" "$OUT/$u.rdc.cubin" && rm -f "$OUT/$u.rdc.cubin" ) &
    pids+=($!)
  fi
done
# the reference's host edge builder and strand loader/resampler (mesh_utils.cpp,
# hair_loader.cpp) behind a small C shim, for the CPU tests
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$OUT/libref_mesh.so" ] || [ "$SRC/mesh_utils.cpp" -nt "$OUT/libref_mesh.so" ] || [ "$HERE/ref_mesh_shim.cpp" -nt "$OUT/libref_mesh.so" ]; then
  ( g++ -O2 -std=c++17 -shared -fPIC -I"$SRC" -o "$OUT/libref_mesh.so" "$SRC/mesh_utils.cpp" "$SRC/hair_loader.cpp" \
        "$HERE/ref_mesh_shim.cpp" ) &
  pids+=($!)
fi
for p in "${pids[@]}"; do wait "$p"; done
echo "build_ref.sh: cubins and libref_mesh.so in $OUT"
