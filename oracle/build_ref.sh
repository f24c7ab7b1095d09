#!/usr/bin/env bash
# Build the reference's CUDA Riemann solver (geoflood_rp2.cu) for the host,
# from the reference tree where it lies, into oracle/_ref/libref_riemann.so.
# Test infrastructure only (pins the oracle). Skips quietly when the
# reference tree is absent (e.g. on a machine without it).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${GF_REFERENCE_ROOT:-/root/reference}"
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
