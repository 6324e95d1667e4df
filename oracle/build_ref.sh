#!/usr/bin/env bash
# Compiles the reference's own device kernels (src/CUDA/cudaEuler2DmixO3RK3/GPUevolve.cu and the
# headers it includes) from the sources where they lie, into cubins under oracle/_ref/.
# TEST INFRASTRUCTURE ONLY: the cubins are the GPU-side oracle that ref_harness.cpp launches.
# Runs where the reference tree is mounted; the cubins then travel with the repository.
set -euo pipefail
REF="${AFAR_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/src/CUDA/cudaEuler2DmixO3RK3"
NVCC="${NVCC:-nvcc}"
if [ ! -f "$SRC/GPUevolve.cu" ]; then
  echo "reference sources not found under $REF; keeping existing cubins" >&2
  exit 0
fi
mkdir -p "$OUT"
for arch in "compute_100,code=sm_100" "compute_103a,code=sm_103a"; do
  tag="${arch##*=}"
  "$NVCC" -cubin -O3 -gencode "arch=$arch" -I"$SRC" -I"$REF/src/CUDA/BCs/2D" "$SRC/GPUevolve.cu" \
    -o "$OUT/ref_${tag}.cubin"
done
echo "built $(ls "$OUT"/ref_*.cubin | tr '\n' ' ')"
