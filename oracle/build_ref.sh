#!/bin/sh
# Builds the reference's CUDA kernels (Florian-BACHO/bats, bats/CudaKernels/CuFiles/**/*.cu), unmodified,
# into device-code fatbins under oracle/_ref/ for the parity harness (oracle/refkern.py).
# TEST INFRASTRUCTURE ONLY: the outputs are the checker, never part of the product.
# One fatbin per source file, because compute_weights_gradient.cu and compute_weights_gradient_old.cu
# export the same kernel symbol. nvcc's defaults (-fmad=true, IEEE division and square root, no
# fast-math) match NVRTC's defaults, which the reference uses through cp.RawKernel with no options.
set -e
REF="${BATS_REFERENCE:-}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
NVCC="${NVCC:-nvcc}"
[ -n "$REF" ] || { echo "set BATS_REFERENCE to a checkout of the reference" >&2; exit 1; }
[ -d "$REF/bats/CudaKernels/CuFiles" ] || { echo "reference not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
pids=""
for f in "$REF"/bats/CudaKernels/CuFiles/*/*.cu; do
  name="$(basename "$f" .cu)"
  "$NVCC" -fatbin -gencode arch=compute_103a,code=sm_103a -w -o "$OUT/$name.fatbin" "$f" &
  pids="$pids $!"
done
for p in $pids; do wait "$p"; done
ls "$OUT"/*.fatbin | wc -l
