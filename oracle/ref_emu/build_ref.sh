#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY: builds oracle/_ref/libref_emu.so, the reference's
# own kernels, radix sort and scene loader compiled for the host CPU from the
# reference tree where it lies (nothing is copied into this repository).
#
#   usage: oracle/ref_emu/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
#
# The reference's wrapper functions launch kernels with <<<...>>>, which g++
# cannot parse, so only the kernel sections of its .cu files are compiled:
# System.cu lines 1-548 (everything before `extern "C"`) and
# radixsort_kernel.cu lines 1-432 (everything before its host RadixSort).
# The line ranges are checked against marker text first.  The sources are
# streamed to g++ on stdin; no intermediate copy is written.
set -euo pipefail
REF_ROOT="${1:-/root/reference}"
SRC="$REF_ROOT/source"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"

if [ ! -f "$SRC/CUDA/System.cu" ]; then
  echo "build_ref: reference sources not found under $SRC" >&2
  exit 1
fi
sed -n '548p' "$SRC/CUDA/System.cu" | grep -q 'END OF KERNEL.CU' || { echo "build_ref: System.cu:548 marker moved" >&2; exit 1; }
sed -n '550p' "$SRC/CUDA/System.cu" | grep -q 'extern "C"' || { echo "build_ref: System.cu:550 marker moved" >&2; exit 1; }
sed -n '434p' "$SRC/CUDA/radixsort_kernel.cu" | grep -q 'extern "C"' || { echo "build_ref: radixsort_kernel.cu:434 marker moved" >&2; exit 1; }

mkdir -p "$OUT"
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
CXX="${CXX:-g++}"
FLAGS=(-O2 -fPIC -ffp-contract=off -std=c++17 -w)
EMU=(-include "$HERE/emu_prelude.h" -I"$HERE" -I"$HERE/shim" -I"$SRC/CUDA" -I"$SRC/external/cutil" -I"$CUDA_INC")

sed -n '1,548p' "$SRC/CUDA/System.cu" |
  "$CXX" "${FLAGS[@]}" -x c++ -DEMU_SHARED_QUAL=static "${EMU[@]}" -c - -o "$TMP/system_kernels.o" &
{ sed -n '1,432p' "$SRC/CUDA/radixsort_kernel.cu"; echo '#endif'; } |
  "$CXX" "${FLAGS[@]}" -x c++ "${EMU[@]}" -c - -o "$TMP/radixsort_kernels.o" &
"$CXX" "${FLAGS[@]}" "${EMU[@]}" -c "$HERE/ref_harness.cpp" -o "$TMP/ref_harness.o" &
SCN=(-I"$HERE/shim" -I"$SRC/pch" -I"$SRC/SPH" -I"$SRC/external" -I"$SRC/external/cutil" -I"$CUDA_INC")
"$CXX" "${FLAGS[@]}" "${SCN[@]}" -c "$SRC/SPH/Scene.cpp" -o "$TMP/Scene.o" &
"$CXX" "${FLAGS[@]}" "${SCN[@]}" -c "$SRC/SPH/Scene_Load.cpp" -o "$TMP/Scene_Load.o" &
"$CXX" "${FLAGS[@]}" "${SCN[@]}" -c "$HERE/scene_harness.cpp" -o "$TMP/scene_harness.o" &
for f in tinyxml tinyxmlparser tinyxmlerror tinystr; do
  "$CXX" "${FLAGS[@]}" -c "$SRC/external/tinyxml/$f.cpp" -o "$TMP/$f.o" &
done
fail=0
for job in $(jobs -p); do wait "$job" || fail=1; done
[ "$fail" = 0 ] || { echo "build_ref: compile failed" >&2; exit 1; }
"$CXX" -shared -o "$OUT/libref_emu.so" "$TMP"/*.o
echo "build_ref: wrote $OUT/libref_emu.so"
