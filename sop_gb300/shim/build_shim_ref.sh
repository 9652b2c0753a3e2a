#!/usr/bin/env bash
# Links the reference program (samchogroup/SOP, the tree given as $1 or
# $SOP_REFERENCE_DIR) over the GB300 engine, without editing a reference
# source:
#   1. the reference's sources compile unchanged (flags of its release build,
#      common.mk:155-171), with the two stand-in headers of oracle/stubs for
#      the CUDA SDK 3.x cutil_inline.h and cudpp.h;
#   2. objcopy --weaken-symbol makes the reference's own definitions of the
#      functions sop_gb300_shim.cu replaces weak, so the shim's definitions
#      win at link time (-fPIC keeps the calls inside sop.cu going through the
#      symbol, where a non-interposable call could be bound early);
#   3. link: the weakened objects, the shim, the CUDPP stand-in (referenced by
#      the reference's own list drivers, which no longer run) and
#      sop_gb300/libsopgpu.so.
# Output: sop_gb300/shim/_build/sop2_gb300.x, which runs the reference's input
# scripts (main, parser, loaders, host energies, observables, writers and
# underdamped_ctrl are the reference's) with every step on the engine.
# Exit 3 when no reference tree is given.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(cd "$here/../.." && pwd)"
ref="${1:-${SOP_REFERENCE_DIR:-}}"
if [ -z "$ref" ] || [ ! -f "$ref/global.h" ]; then
  echo "build_shim_ref: no reference tree given (argument or SOP_REFERENCE_DIR)" >&2
  exit 3
fi
ref="$(cd "$ref" && pwd)"
out="$here/_build"
mkdir -p "$out"
NVCC="${NVCC:-nvcc}"
arch=(-gencode arch=compute_103a,code=sm_103a)
base=(-O2 -w -DUNIX "${arch[@]}" -Xcompiler -fPIC -Xcompiler -fno-strict-aliasing
      -I "$root/oracle/stubs" -I "$ref")
pids=()
for src in global.cpp param.cpp io.cpp misc.cpp random_generator.cpp; do
  "$NVCC" -std=c++14 "${base[@]}" -x cu -c "$ref/$src" -o "$out/${src%.cpp}.o" & pids+=($!)
done
for src in energy.cu GPUvars.cu sop.cu; do
  "$NVCC" -std=c++14 "${base[@]}" -c "$ref/$src" -o "$out/${src%.cu}.o" & pids+=($!)
done
"$NVCC" -std=c++17 "${base[@]}" -c "$root/oracle/ref_cudpp_cub.cu" -o "$out/cudpp_cub.o" & pids+=($!)
"$NVCC" -std=c++14 "${base[@]}" -I "$root/include" -c "$here/sop_gb300_shim.cu" \
  -o "$out/shim.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
objcopy --weaken-symbol=_Z20update_neighbor_listv --weaken-symbol=_Z16update_pair_listv \
        --weaken-symbol=_Z16update_cell_listv --weaken-symbol=_Z18update_hybrid_listv \
        --weaken-symbol=_Z21underdamped_iterationv "$out/sop.o"
objcopy --weaken-symbol=_Z12clear_forcesv --weaken-symbol=_Z10force_evalv \
        --weaken-symbol=_Z12random_forcev "$out/energy.o"
objcopy --weaken-symbol=_Z16alloc_GPU_arraysv --weaken-symbol=_Z11alloc_cudppv \
        --weaken-symbol=_Z9setup_rngyy "$out/GPUvars.o"
"$NVCC" "${arch[@]}" -o "$out/sop2_gb300.x" "$out/shim.o" "$out/global.o" "$out/param.o" \
  "$out/io.o" "$out/misc.o" "$out/random_generator.o" "$out/energy.o" "$out/GPUvars.o" \
  "$out/sop.o" "$out/cudpp_cub.o" -L "$root/sop_gb300" -lsopgpu \
  -Xlinker -rpath -Xlinker "$root/sop_gb300"
echo "build_shim_ref: $out/sop2_gb300.x (from $ref)"
