#!/usr/bin/env bash
# Build the reference's CUDA Riemann solver (geoflood_rp2.cu) and its CUDA
# patch update (cudaclaw_flux2.cu with cudaclaw_limiters.cu and
# geoflood_src2.cu) for the host, from the reference tree where they lie,
# into oracle/_ref/libref_riemann.so and oracle/_ref/libref_patch.so.
# Test infrastructure only (pins the oracle). The reference tree is the
# first argument, else GF_REFERENCE_ROOT, else the checkout this recipe was
# written against; where none of them holds the sources the script skips
# quietly (the GPU machines have no reference tree).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${GF_REFERENCE_ROOT:-/root/reference}}"
SRC="$REF/src/fc2d_cpu_cuda"
OUT="$HERE/_ref"
if [ ! -f "$SRC/riemann_source/geoflood_rp2.cu" ]; then
    echo "build_ref: reference tree not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT/stub"
# ForestClaw headers the file includes but does not use: empty stand-ins.
for h in fclaw2d_clawpatch.h fclaw2d_clawpatch_options.h fclaw2d_include_all.h; do
    : > "$OUT/stub/$h"
done
CXX="${CXX:-g++}"
FLAGS=(-O2 -ffp-contract=off -fno-fast-math -fPIC -std=c++17 -w
       -include "$HERE/ref_shim.h" -DFC2D_CPUCUDA_H
       -I"$OUT/stub" -I"$SRC" -I"$SRC/riemann_source")
"$CXX" "${FLAGS[@]}" -x c++ -c "$SRC/riemann_source/geoflood_rp2.cu" -o "$OUT/geoflood_rp2.o"
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_riemann_pin.cpp" -o "$OUT/ref_riemann_pin.o"
"$CXX" -shared -o "$OUT/libref_riemann.so" "$OUT/geoflood_rp2.o" "$OUT/ref_riemann_pin.o" -lm
echo "build_ref: built $OUT/libref_riemann.so"

# The patch update: one host thread per patch (ref_shim_patch.h), the CUB
# block reduction and the thrust include replaced by stand-ins.
mkdir -p "$OUT/stub/cub/block" "$OUT/stub/thrust"
: > "$OUT/stub/thrust/device_vector.h"
cat > "$OUT/stub/cub/block/block_reduce.cuh" <<'CUB'
/* one-thread stand-in for cub::BlockReduce (host build of the reference) */
#pragma once
namespace cub {
struct Max {};
template <class T, int N>
struct BlockReduce {
    struct TempStorage {};
    explicit BlockReduce(TempStorage&) {}
    T Reduce(T v, Max) { return v; }
};
}
CUB
PFLAGS=(-O2 -ffp-contract=off -fno-fast-math -fPIC -std=c++17 -w
        -include "$HERE/ref_shim_patch.h" -DFC2D_CPUCUDA_H
        -I"$HERE" -I"$OUT/stub" -I"$SRC" -I"$SRC/riemann_source")
"$CXX" "${PFLAGS[@]}" -x c++ -c "$SRC/riemann_source/geoflood_rp2.cu" -o "$OUT/p_rp2.o"
"$CXX" "${PFLAGS[@]}" -x c++ -c "$SRC/riemann_source/geoflood_src2.cu" -o "$OUT/p_src2.o"
"$CXX" "${PFLAGS[@]}" -x c++ -c "$SRC/cuda_source/cudaclaw_limiters.cu" -o "$OUT/p_limiters.o"
"$CXX" "${PFLAGS[@]}" -c "$HERE/ref_patch_pin.cpp" -o "$OUT/p_flux2.o"
"$CXX" -shared -o "$OUT/libref_patch.so" "$OUT/p_rp2.o" "$OUT/p_src2.o" "$OUT/p_limiters.o" \
    "$OUT/p_flux2.o" -lm
echo "build_ref: built $OUT/libref_patch.so"
