#!/bin/sh
# ORACLE recipe (test infrastructure only): compile the reference's own, unmodified CUDA
# kernels (GPU/dipole_GPU.cu of GAIN-MPI) for sm_103a into a device-only cubin under
# oracle/_ref/.  Runs where the reference tree is present; nothing is copied from it.
# oracle/ref_harness.cu loads this cubin through the CUDA driver API on the GPU machine.
set -e
REF=${GAIN_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_ref"
if [ ! -f "$REF/GPU/dipole_GPU.cu" ]; then
    echo "reference tree not found at $REF; keeping any prebuilt cubin" >&2
    exit 0
fi
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo \
     -I"$REF/GPU" -o "$HERE/_ref/dipole_GPU.cubin.tmp" "$REF/GPU/dipole_GPU.cu" 2> "$HERE/_ref/build.log"
mv "$HERE/_ref/dipole_GPU.cubin.tmp" "$HERE/_ref/dipole_GPU.cubin"
echo "built $HERE/_ref/dipole_GPU.cubin"
