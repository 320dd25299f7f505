#!/usr/bin/env bash
# Build the reference's own voxelizer code into oracle/_ref/.
# Test infrastructure only: these builds are the checker and the timed reference baseline, never
# part of the product.  Outputs go only into oracle/_ref/ (git-ignored, shipped to the GPU machine
# with the repository snapshot); nothing of the reference is committed.
#
#   src/                      the reference CPU voxelizer's and command-line program's own source
#                             files, staged unmodified from the reference tree (src/cpu_voxelizer.
#                             {cpp,h}, main.cpp, util.h, util_io.{cpp,h}, util_cuda.{cpp,h}, timer.h,
#                             morton_LUTs.h, libs/cuda/*, libs/magicavoxel_file_writer/VoxWriter.*)
#                             so that machines without the reference tree (the Arm GPU host) can
#                             build them too
#   libref_cpu.so             src/cpu_voxelizer.cpp (OpenMP CPU voxelizer) + oracle/ref_cpu_shim.cpp,
#                             compiled from the staged copy for the machine that runs this script
#   cuda_voxelizer_relinked   the reference's command-line program (src/main.cpp with its I/O and
#                             CUDA-init helpers) linked against this repository's libcvx.so in place
#                             of src/voxelize.cu and src/voxelize_solid.cu, as INTEGRATION.md
#                             describes; built from the staged copy where libcvx.so exists
#   libref_io.so              src/util_io.cpp (output writers) + VoxWriter + oracle/ref_io_shim.cpp,
#                             host code (golden-file generation; only where the reference tree is)
#   ref_voxelize.cubin        src/voxelize.cu        (kernel voxelize_triangle) for sm_103a
#   ref_voxelize_solid.cubin  src/voxelize_solid.cu  (kernel voxelize_triangle_solid) for sm_103a
#
# The cubins are device code: oracle/ref_gpu_runner.cu loads them with the CUDA driver API on the
# GPU machine.  They are compiled the way the reference's CMake build compiles them
# (CMakeLists.txt:46-62: no fast-math, default --fmad=true, device -O3), only with the
# architecture set to sm_103a.
#
# Usage: oracle/build_ref.sh REFERENCE_ROOT   stage and build everything from the reference tree
#        oracle/build_ref.sh --staged         build libref_cpu.so from oracle/_ref/src only
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
CUDA_HOME="${CUDA_HOME:-/usr/local/cuda}"
NVCC="$CUDA_HOME/bin/nvcc"
if [ $# -ne 1 ]; then
  echo "usage: $0 REFERENCE_ROOT | --staged" >&2
  exit 2
fi
mkdir -p "$OUT"

build_main() {
  # The reference's main.cpp, unmodified, calling voxelize()/voxelize_solid() from libcvx.so.
  local LIB="$HERE/../cuda_voxelizer_gb300/_lib"
  if [ ! -f "$LIB/libcvx.so" ]; then
    echo "build_ref: libcvx.so not built; skipping the relinked command-line program" >&2
    return 0
  fi
  "$NVCC" -O2 -std=c++17 -w -cudart shared -Xcompiler -fopenmp -Xcompiler -ffp-contract=off \
      -I"$HERE/trimesh_shim" -I"$SRC" \
      "$SRC/main.cpp" "$SRC/util_io.cpp" "$SRC/util_cuda.cpp" "$SRC/cpu_voxelizer.cpp" \
      "$SRC/libs/magicavoxel_file_writer/VoxWriter.cpp" \
      -L"$LIB" -lcvx -Xlinker -rpath,"$LIB" -lgomp -o "$OUT/cuda_voxelizer_relinked"
}

build_cpu() {
  # Reference CPU path.  -O2 stands in for a Release build (the CMake file sets no build type).
  # -ffp-contract=off: the reference's x86-64 build has no FMA, so a*b+c is never contracted there;
  # gcc on aarch64 would contract it by default and change the results.
  g++ -O2 -fopenmp -std=c++17 -fPIC -shared -w -ffp-contract=off \
      -I"$HERE/trimesh_shim" -I"$SRC" -I"$CUDA_HOME/include" \
      "$HERE/ref_cpu_shim.cpp" "$SRC/cpu_voxelizer.cpp" \
      -o "$OUT/libref_cpu.so"
}

if [ "$1" = "--staged" ]; then
  if [ ! -f "$SRC/cpu_voxelizer.cpp" ]; then
    echo "build_ref: no staged reference sources in $SRC; skipping" >&2
    exit 0
  fi
  build_cpu
  if [ -f "$SRC/main.cpp" ]; then build_main || echo "build_ref: relinked command-line program not built" >&2; fi
  echo "build_ref: wrote libref_cpu.so and the relinked command-line program from the staged sources"
  exit 0
fi

REF="$1"
if [ ! -f "$REF/src/cpu_voxelizer.cpp" ]; then
  echo "build_ref: reference sources not found under $REF; skipping" >&2
  exit 0
fi
mkdir -p "$SRC/libs/cuda" "$SRC/libs/magicavoxel_file_writer"
for f in cpu_voxelizer.cpp cpu_voxelizer.h util.h timer.h morton_LUTs.h libs/cuda/helper_math.h \
         main.cpp util_io.cpp util_io.h util_cuda.cpp util_cuda.h libs/cuda/helper_cuda.h libs/cuda/helper_string.h \
         libs/magicavoxel_file_writer/VoxWriter.cpp libs/magicavoxel_file_writer/VoxWriter.h; do
  cp "$REF/src/$f" "$SRC/$f"
done

build_cpu &
pid_cpu=$!
(build_main || echo "build_ref: relinked command-line program not built" >&2) &
pid_main=$!

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
wait $pid_main
wait $pid_io
wait $pid_s
wait $pid_d
echo "build_ref: wrote $(ls "$OUT" | tr '\n' ' ')"
