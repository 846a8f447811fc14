#!/usr/bin/env bash
# Build the reference's own CUDA kernels (device code only) into oracle/_ref/ as
# sm_103a cubins, straight from the reference sources where they lie.
#
# Test infrastructure only: the cubins are driven by oracle/refharness.cpp on a
# GPU machine to produce the golden records that pin the CPU oracle.  Nothing in
# the product loads them.  The reference's host code is not compiled (it would be
# x86 code here; the GPU machine is aarch64); refharness.cpp restates the host
# loop instead and launches the reference kernels through the CUDA driver API.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   default: $A3D_REFERENCE, else a checkout named "reference" beside this repository
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${A3D_REFERENCE:-$HERE/../../reference}}
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
if [ ! -d "$REF/src" ]; then
  echo "build_ref.sh: reference sources not found under $REF/src" >&2
  exit 2
fi
mkdir -p "$OUT"
build() {  # $1 = source file name, $2 = output stem
  "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -o "$OUT/$2.cubin" "$REF/src/$1"
}
build Toa_3dfd_cuda.cu                    ref_2order &
build Toa_gpu_3diso_fd_1orderfunciton.cu  ref_1order &
build Toa_gpu_3dvti_fd_1orderfunciton.cu  ref_vti &
build Toa_gpu_3dtti_fd_1orderfunciton.cu  ref_tti &
wait
ls -l "$OUT"
