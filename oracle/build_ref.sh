#!/usr/bin/env bash
# Builds oracle/_ref/libsopref.so from the reference's own, unmodified sources
# where they lie (default /root/reference, or $SOP_REFERENCE_DIR), plus the
# two stub headers in oracle/stubs and the C-ABI harness oracle/ref_harness.cpp.
# Test infrastructure only: the library pins the oracle against the
# reference's host routines.  Exits 0 without building when the reference
# sources are absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${SOP_REFERENCE_DIR:-/root/reference}"
out="$here/_ref"
if [ ! -f "$ref/energy.cu" ]; then
  echo "build_ref: reference sources not found at $ref; skipping" >&2
  exit 0
fi
mkdir -p "$out"
NVCC="${NVCC:-nvcc}"
flags=(-O2 -std=c++14 -w -Xcompiler -fPIC -Xcompiler -ffp-contract=off
       -gencode arch=compute_103a,code=sm_103a -I "$here/stubs" -I "$ref")
pids=()
for src in global.cpp param.cpp io.cpp misc.cpp random_generator.cpp; do
  "$NVCC" "${flags[@]}" -x cu -c "$ref/$src" -o "$out/${src%.cpp}.o" & pids+=($!)
done
for src in energy.cu GPUvars.cu sop.cu; do
  "$NVCC" "${flags[@]}" -c "$ref/$src" -o "$out/${src%.cu}.o" & pids+=($!)
done
"$NVCC" "${flags[@]}" -x cu -c "$here/ref_harness.cpp" -o "$out/ref_harness.o" & pids+=($!)
"$NVCC" "${flags[@]}" -c "$here/ref_cudpp_stub.cpp" -o "$out/ref_cudpp_stub.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -shared -gencode arch=compute_103a,code=sm_103a -o "$out/libsopref.so" "$out"/*.o
echo "build_ref: $out/libsopref.so"
