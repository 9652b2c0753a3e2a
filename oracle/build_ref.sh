#!/usr/bin/env bash
# Builds the reference's own code into oracle/_ref from its unmodified sources,
# where they lie, in the tree given as $1 (or $SOP_REFERENCE_DIR):
#
#   libsopref.so      host routines, sop.cu with its host list filters
#                     (through ref_sop_cpu_lists.cu) and the C-ABI harness
#                     ref_harness.cpp; its host entry points run without a GPU
#   libsopref_gpu.so  the same with sop.cu as it ships: CUDPP-based GPU list
#                     drivers (CUDPP stand-in ref_cudpp_cub.cu), force kernels,
#                     cuRAND noise; needs a GPU
#   sop2ref.x         the reference program itself (main() of sop.cu) over the
#                     same objects as libsopref_gpu.so
#   sop2ref_hostrng.x the same program built with its host noise generator
#                     instead of cuRAND (USE_CURAND taken back, through
#                     ref_energy_hostrng.cu and ref_sop_hostrng.cu)
#
# Every artefact links with the wrappers of ref_link_wraps.cpp (host-side
# copies for the host filters, an optional cuRAND seed from the environment).
# The two stub headers in oracle/stubs stand in for the CUDA SDK 3.x
# cutil_inline.h and cudpp.h.  Flags follow the reference's release build
# (common.mk:155-171: -O2 -DUNIX -fno-strict-aliasing, default nvcc math);
# host code adds -ffp-contract=off so aarch64 hosts compute the FP32 list
# predicates exactly as x86-64 hosts do.
#
# TEST INFRASTRUCTURE ONLY.  Exits 0 without building when no tree is given
# or the tree holds no reference sources.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-${SOP_REFERENCE_DIR:-}}"
out="$here/_ref"
if [ -z "$ref" ] || [ ! -f "$ref/energy.cu" ]; then
  echo "build_ref: no reference tree given (argument or SOP_REFERENCE_DIR); skipping" >&2
  exit 0
fi
ref="$(cd "$ref" && pwd)"
mkdir -p "$out/obj"
NVCC="${NVCC:-nvcc}"
arch=(-gencode arch=compute_103a,code=sm_103a)
base=(-O2 -w -DUNIX "${arch[@]}"
      -Xcompiler -fPIC -Xcompiler -fno-strict-aliasing -Xcompiler -ffp-contract=off
      -I "$here/stubs" -I "$ref")
flags=(-std=c++14 "${base[@]}")
o="$out/obj"
pids=()
for src in global.cpp param.cpp io.cpp misc.cpp random_generator.cpp; do
  "$NVCC" "${flags[@]}" -x cu -c "$ref/$src" -o "$o/${src%.cpp}.o" & pids+=($!)
done
for src in energy.cu GPUvars.cu sop.cu; do
  "$NVCC" "${flags[@]}" -c "$ref/$src" -o "$o/${src%.cu}.o" & pids+=($!)
done
"$NVCC" "${flags[@]}" -c "$here/ref_sop_cpu_lists.cu" -o "$o/sop_cpu_lists.o" & pids+=($!)
"$NVCC" "${flags[@]}" -c "$here/ref_energy_hostrng.cu" -o "$o/energy_hostrng.o" & pids+=($!)
"$NVCC" "${flags[@]}" -c "$here/ref_sop_hostrng.cu" -o "$o/sop_hostrng.o" & pids+=($!)
"$NVCC" "${flags[@]}" -x cu -c "$here/ref_harness.cpp" -o "$o/ref_harness.o" & pids+=($!)
"$NVCC" -std=c++17 "${base[@]}" -c "$here/ref_cudpp_cub.cu" -o "$o/ref_cudpp_cub.o" & pids+=($!)
"$NVCC" "${flags[@]}" -x cu -c "$here/ref_link_wraps.cpp" -o "$o/ref_link_wraps.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
common=("$o/global.o" "$o/param.o" "$o/io.o" "$o/misc.o" "$o/random_generator.o"
        "$o/energy.o" "$o/GPUvars.o" "$o/ref_cudpp_cub.o" "$o/ref_link_wraps.o")
wraps=(-Xlinker --wrap=cudaMemcpy -Xlinker --wrap=_Z9setup_rngyy)
# -Bsymbolic: the reference's globals have names that the C library also
# exports (GPUvars.cu's `err` is glibc's err(3)); a library loaded into a host
# process must bind them to its own definitions, as the reference's program does
shared=(-shared -Xlinker -Bsymbolic)
"$NVCC" "${shared[@]}" "${arch[@]}" "${wraps[@]}" -o "$out/libsopref.so" \
  "${common[@]}" "$o/sop_cpu_lists.o" "$o/ref_harness.o" & l1=$!
"$NVCC" "${shared[@]}" "${arch[@]}" "${wraps[@]}" -o "$out/libsopref_gpu.so" \
  "${common[@]}" "$o/sop.o" "$o/ref_harness.o" & l2=$!
"$NVCC" "${arch[@]}" "${wraps[@]}" -o "$out/sop2ref.x" "${common[@]}" "$o/sop.o" & l3=$!
hostrng=()
for f in "${common[@]}"; do [ "$f" = "$o/energy.o" ] || hostrng+=("$f"); done
"$NVCC" "${arch[@]}" "${wraps[@]}" -o "$out/sop2ref_hostrng.x" "${hostrng[@]}" \
  "$o/energy_hostrng.o" "$o/sop_hostrng.o" & l4=$!
wait $l1; wait $l2; wait $l3; wait $l4
echo "build_ref: $out/libsopref.so $out/libsopref_gpu.so $out/sop2ref.x $out/sop2ref_hostrng.x (from $ref)"
