#!/usr/bin/env bash
# Builds the reference checker: the reference project's own LBM sources
# (src/LBM/*.cpp, compiled unchanged) against the project-written AMReX
# stand-in in oracle/ref_shim/, plus oracle/ref_driver.cpp, into
#   oracle/_ref/libmphref2d.so  (AMREX_SPACEDIM=2: D2Q9)
#   oracle/_ref/libmphref3d.so  (AMREX_SPACEDIM=3: D3Q15, D3Q19, D3Q27)
# with OpenMP, so the reference's `#pragma omp parallel` MFIter loops run on
# every host thread (the reference arm of bench.py times them).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $MPH_REFERENCE_ROOT, else /root/reference.
# Where the reference checkout is present, its src/LBM directory is also
# copied into baseline/_ref/src/LBM (git-ignored, never committed) so that a
# machine without the checkout (the Arm GPU host) builds the same sources
# from there; the build compiles the checkout when present, else that copy.
# Exits 0 without building when neither exists.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
repo="$(cd "$here/.." && pwd)"
ref="${1:-${MPH_REFERENCE_ROOT:-/root/reference}}"
staged="$repo/baseline/_ref/src"
if [ -f "$ref/src/LBM/Collision.cpp" ]; then
    src="$ref/src"
    mkdir -p "$staged"
    rm -rf "$staged/LBM.tmp"
    cp -r "$src/LBM" "$staged/LBM.tmp"
    rm -rf "$staged/LBM"
    mv "$staged/LBM.tmp" "$staged/LBM"
elif [ -f "$staged/LBM/Collision.cpp" ]; then
    src="$staged"
else
    echo "build_ref: reference sources not found under $ref or $staged; skipping" >&2
    exit 0
fi
out="$here/_ref"
mkdir -p "$out"
cxx="${CXX:-g++}"
# -O3 as AMReX's GNU make (COMP=gnu, DEBUG=FALSE) builds the reference, with
# GCC's complete-peeling limits raised: the reference's per-population loops
# (9-27 iterations) index constexpr lattice tables that fold to constants only
# once a loop is fully unrolled; at GCC's default limits the tables are
# rebuilt on every call and the step runs ~6x slower per core.  Unrolling does
# not reassociate floating point, so the results keep their bits.
flags=(-O3 --param max-completely-peel-times=40 --param max-completely-peeled-insns=8000
       -std=c++17 -fPIC -shared -fopenmp -ffp-contract=off -w
       -I"$here/ref_shim" -I"$here" -I"$src" -I"$src/LBM")
srcs=("$src/LBM/Collision.cpp" "$src/LBM/Streaming.cpp" "$src/LBM/Macroscopic.cpp"
      "$src/LBM/Equilibrium.cpp" "$src/LBM/BoundaryConditions.cpp" "$src/LBM/Units.cpp"
      "$here/ref_driver.cpp")
"$cxx" "${flags[@]}" -DAMREX_SPACEDIM=2 "${srcs[@]}" -o "$out/libmphref2d.so.tmp" &
p2=$!
"$cxx" "${flags[@]}" -DAMREX_SPACEDIM=3 "${srcs[@]}" -o "$out/libmphref3d.so.tmp" &
p3=$!
wait "$p2"
wait "$p3"
mv "$out/libmphref2d.so.tmp" "$out/libmphref2d.so"
mv "$out/libmphref3d.so.tmp" "$out/libmphref3d.so"
echo "build_ref: built $out/libmphref2d.so $out/libmphref3d.so from $src"
