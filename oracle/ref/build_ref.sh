#!/bin/bash
# ORACLE build recipe: compile the reference's own CUDA kernels into cubins.
#
# Reads the reference sources from REF_SRC (default /root/reference/src) and
# writes only into oracle/_ref/.  Run where the reference tree exists; the
# cubins are device code and travel to the GPU machine with the repository.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
out="$here/../_ref"
REF_SRC="${REF_SRC:-/root/reference/src}"
NVCC="${NVCC:-nvcc}"
if [ ! -f "$REF_SRC/rungeKutta.cu" ]; then
    echo "build_ref.sh: reference sources not found at $REF_SRC; skipping" >&2
    exit 0
fi
mkdir -p "$out"
for prec in 64 32; do
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -DPRECISION=$prec \
        -I"$REF_SRC" -diag-suppress 177,550 -w \
        "$here/ref_kernels.cu" -o "$out/glemur_ref$prec.cubin" &
done
wait
ls -l "$out"/glemur_ref*.cubin
