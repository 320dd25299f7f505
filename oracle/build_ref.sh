#!/usr/bin/env bash
# Build the reference's own voxelizer code, from its sources where they lie, into oracle/_ref/.
# Test infrastructure only: these builds are the checker and the timed reference baseline,
# never part of the product.  Nothing is copied out of the reference tree; outputs go only
# into oracle/_ref/ (git-ignored, shipped to the GPU machine with the repository snapshot).
#
#   libref_cpu.so             src/cpu_voxelizer.cpp (OpenMP CPU voxelizer) + oracle/ref_cpu_shim.cpp,
#                             host-architecture code, so it is only usable where it was built.
#   libref_io.so              src/util_io.cpp (output writers) + VoxWriter + oracle/ref_io_shim.cpp,
#                             host-architecture code (golden-file generation)
#   ref_voxelize.cubin        src/voxelize.cu        (kernel voxelize_triangle) for sm_103a
#   ref_voxelize_solid.cubin  src/voxelize_solid.cu  (kernel voxelize_triangle_solid) for sm_103a
#
# The cubins are device code: oracle/ref_gpu_runner.cu loads them with the CUDA driver API on the
# GPU machine.  They are compiled the way the reference's CMake build compiles them
# (CMakeLists.txt:46-62: no fast-math, default --fmad=true, device -O3), only with the
# architecture set to sm_103a.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ ! -f "$REF/src/cpu_voxelizer.cpp" ]; then
  echo "build_ref: reference sources not found under $REF; skipping" >&2
  exit 0
fi
CUDA_HOME="${CUDA_HOME:-/usr/local/cuda}"
NVCC="$CUDA_HOME/bin/nvcc"

# Reference CPU path.  -O2 stands in for a Release build (the CMake file sets no build type);
# the x86-64 baseline has no FMA, so gcc cannot contract a*b+c here.
g++ -O2 -fopenmp -std=c++17 -fPIC -shared -w \
    -I"$HERE/trimesh_shim" -I"$REF/src" -I"$CUDA_HOME/include" \
    "$HERE/ref_cpu_shim.cpp" "$REF/src/cpu_voxelizer.cpp" \
    -o "$OUT/libref_cpu.so" &
pid_cpu=$!

# Reference output writers (src/util_io.cpp with its vendored MagicaVoxel writer), host code.
g++ -O2 -std=c++17 -fPIC -shared -w -DSILENT \
    -I"$HERE/trimesh_shim" -I"$REF/src" -I"$CUDA_HOME/include" \
    "$HERE/ref_io_shim.cpp" "$REF/src/util_io.cpp" "$REF/src/libs/magicavoxel_file_writer/VoxWriter.cpp" \
    -o "$OUT/libref_io.so" &
pid_io=$!

# Reference GPU kernels for sm_103a, device code only.
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -w \
    -I"$HERE/trimesh_shim" -I"$REF/src" \
    "$REF/src/voxelize.cu" -o "$OUT/ref_voxelize.cubin" &
pid_s=$!
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -w \
    -I"$HERE/trimesh_shim" -I"$REF/src" \
    "$REF/src/voxelize_solid.cu" -o "$OUT/ref_voxelize_solid.cubin" &
pid_d=$!

wait $pid_cpu
wait $pid_io
wait $pid_s
wait $pid_d
echo "build_ref: wrote $(ls "$OUT" | tr '\n' ' ')"
