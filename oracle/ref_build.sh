#!/usr/bin/env bash
# Build recipe for the reference-kernel oracle (test infrastructure only).
# Compiles the reference's SDGC kernel headers, where they lie in the
# reference tree, into device code under oracle/_ref/ (git-ignored):
#   oracle/_ref/sdgc_ref.cubin   sm_103a cubin
# No reference source is copied.  Usage: oracle/ref_build.sh [REFERENCE_ROOT]
# (the root is the argument, else $SNICIT_REFERENCE_ROOT, else the reference
# mount of the build container, /root/reference)
set -euo pipefail
REF="${1:-${SNICIT_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
if [ ! -d "$REF/src/SDGC" ]; then
  echo "reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
FLAGS=(-std=c++17 --extended-lambda -O3 -w -I "$REF/src/SDGC" -I "$REF/3rd-party")
"$NVCC" "${FLAGS[@]}" -cubin -gencode arch=compute_103a,code=sm_103a \
  "$HERE/ref_kernels.cu" -o "$OUT/sdgc_ref.cubin"
echo "$OUT/sdgc_ref.cubin"
