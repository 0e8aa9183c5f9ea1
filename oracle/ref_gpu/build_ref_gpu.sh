#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY: compiles the reference's own CUDA kernels for the
# GB300 from the reference tree where it lies, into oracle/_ref/:
#   ref_system.ptx, ref_system_fast.ptx   System.cu lines 1-548 (the kernels,
#                                          everything before `extern "C"`)
#   ref_radix.ptx                          radixsort_kernel.cu lines 1-432
#   ref_gpu_entries.txt                    the kernels' entry names, from
#                                          ptxas -v (name=entry)
# `ref_system.ptx` is built with --fmad=false, like the host build in
# oracle/ref_emu (-ffp-contract=off), for parity; `ref_system_fast.ptx` with
# nvcc's defaults, as the reference's own build would be, for timing.  The
# harness oracle/ref_gpu/ref_gpu.cpp loads them through the CUDA driver API.
# The kernel sections are written to a temporary directory for nvcc, which is
# removed afterwards; nothing is copied into this repository.
#
#   usage: oracle/ref_gpu/build_ref_gpu.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF_ROOT="${1:-/root/reference}"
SRC="$REF_ROOT/source"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
NVCC="${NVCC:-${CUDA_HOME:-/usr/local/cuda}/bin/nvcc}"

if [ ! -f "$SRC/CUDA/System.cu" ]; then
  echo "build_ref_gpu: reference sources not found under $SRC" >&2
  exit 1
fi
sed -n '548p' "$SRC/CUDA/System.cu" | grep -q 'END OF KERNEL.CU' || { echo "build_ref_gpu: System.cu:548 marker moved" >&2; exit 1; }
sed -n '434p' "$SRC/CUDA/radixsort_kernel.cu" | grep -q 'extern "C"' || { echo "build_ref_gpu: radixsort_kernel.cu:434 marker moved" >&2; exit 1; }

mkdir -p "$OUT"
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
sed -n '1,548p' "$SRC/CUDA/System.cu" > "$TMP/system_kernels.cu"
{ sed -n '1,432p' "$SRC/CUDA/radixsort_kernel.cu"; echo '#endif'; } > "$TMP/radix_kernels.cu"
INC=(-include "$HERE/gpu_prelude.h" -I"$HERE/../ref_emu/shim" -I"$SRC/CUDA" -I"$SRC/external/cutil")
ARCH=(-gencode arch=compute_103a,code=sm_103a)
FLAGS=(-std=c++17 -w)

"$NVCC" "${FLAGS[@]}" "${INC[@]}" -arch=compute_103a --fmad=false -ptx "$TMP/system_kernels.cu" -o "$OUT/ref_system.ptx" &
"$NVCC" "${FLAGS[@]}" "${INC[@]}" -arch=compute_103a -ptx "$TMP/system_kernels.cu" -o "$OUT/ref_system_fast.ptx" &
"$NVCC" "${FLAGS[@]}" "${INC[@]}" -arch=compute_103a -ptx "$TMP/radix_kernels.cu" -o "$OUT/ref_radix.ptx" &
# entry names as ptxas reports them (the throwaway cubins stay in $TMP)
"$NVCC" "${FLAGS[@]}" "${INC[@]}" "${ARCH[@]}" -Xptxas -v -cubin "$TMP/system_kernels.cu" -o "$TMP/s.cubin" > "$TMP/s.log" 2>&1 &
"$NVCC" "${FLAGS[@]}" "${INC[@]}" "${ARCH[@]}" -Xptxas -v -cubin "$TMP/radix_kernels.cu" -o "$TMP/r.cubin" > "$TMP/r.log" 2>&1 &
fail=0
for job in $(jobs -p); do wait "$job" || fail=1; done
[ "$fail" = 0 ] || { cat "$TMP"/*.log >&2; echo "build_ref_gpu: compile failed" >&2; exit 1; }

{
  for k in integrateD calcHashD reorderD computeDensityD computeForceD RadixSum RadixPrefixSum RadixAddOffsetsAndShuffle; do
    e=$(grep -ho "Compiling entry function '[^']*'" "$TMP/s.log" "$TMP/r.log" | sed "s/Compiling entry function '\(.*\)'/\1/" |
        grep -E "^_Z[0-9]+${k}[A-Z]|^_Z[0-9]+${k}v$" | head -1)
    [ -n "$e" ] || { echo "build_ref_gpu: no entry for $k" >&2; exit 1; }
    echo "$k=$e"
  done
} > "$OUT/ref_gpu_entries.txt"
echo "build_ref_gpu: wrote $OUT/ref_system.ptx ref_system_fast.ptx ref_radix.ptx ref_gpu_entries.txt"
