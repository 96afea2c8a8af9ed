#!/usr/bin/env bash
# Builds the reference checker: the reference project's own LBM sources
# (src/LBM/*.cpp, compiled unchanged where they lie) against the project-written
# AMReX stand-in in oracle/ref_shim/, plus oracle/ref_driver.cpp, into
#   oracle/_ref/libmphref2d.so  (AMREX_SPACEDIM=2: D2Q9)
#   oracle/_ref/libmphref3d.so  (AMREX_SPACEDIM=3: D3Q15, D3Q19, D3Q27)
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Exits 0 without building when the reference sources are absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-/root/reference}"
src="$ref/src"
if [ ! -f "$src/LBM/Collision.cpp" ]; then
    echo "build_ref: reference sources not found under $ref; skipping" >&2
    exit 0
fi
out="$here/_ref"
mkdir -p "$out"
cxx="${CXX:-g++}"
flags=(-O2 -std=c++17 -fPIC -shared -ffp-contract=off -w
       -I"$here/ref_shim" -I"$here" -I"$src" -I"$src/LBM")
srcs=("$src/LBM/Collision.cpp" "$src/LBM/Streaming.cpp" "$src/LBM/Macroscopic.cpp"
      "$src/LBM/Equilibrium.cpp" "$src/LBM/BoundaryConditions.cpp" "$src/LBM/Units.cpp"
      "$here/ref_driver.cpp")
"$cxx" "${flags[@]}" -DAMREX_SPACEDIM=2 "${srcs[@]}" -o "$out/libmphref2d.so" &
p2=$!
"$cxx" "${flags[@]}" -DAMREX_SPACEDIM=3 "${srcs[@]}" -o "$out/libmphref3d.so" &
p3=$!
wait "$p2"
wait "$p3"
echo "build_ref: built $out/libmphref2d.so $out/libmphref3d.so"
