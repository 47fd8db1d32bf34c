#!/usr/bin/env bash
# Build oracle/_ref/ref_track_sm103a.cubin: the reference's own CUDA tracking
# and remap kernels, compiled from the reference sources where they lie
# (REF_ROOT, default /root/reference) for sm_103a.
#
# TEST INFRASTRUCTURE ONLY.  Device code only (a cubin), so the result runs
# on any host architecture through the CUDA driver API (oracle/ref_cuda.py).
# Flags follow the reference's release CUDA build (sixtracklib/cuda/
# CMakeLists.txt: -fmad=false -lineinfo -D_FORCE_INLINES, _GPUCODE=1); the
# configuration headers are the ones oracle/build_ref.sh writes (the
# reference's default feature values).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_ROOT/sixtracklib/cuda/kernels/track_particles.cu" ]; then
    echo "reference CUDA sources not found under $REF_ROOT" >&2
    exit 2
fi
if [ ! -f "$OUT/include/sixtracklib/common/generated/config.h" ]; then
    "$HERE/build_ref.sh" > /dev/null
fi
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -fmad=false -lineinfo \
    -D_FORCE_INLINES -D_GPUCODE=1 -w \
    -I "$OUT/include" -I "$REF_ROOT" \
    "$HERE/ref_cuda_kernels.cu" -o "$OUT/ref_track_sm103a.cubin.tmp"
mv "$OUT/ref_track_sm103a.cubin.tmp" "$OUT/ref_track_sm103a.cubin"
echo "built $OUT/ref_track_sm103a.cubin"
