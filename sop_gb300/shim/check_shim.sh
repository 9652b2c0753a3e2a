#!/usr/bin/env bash
# Compiles the reference-side shim (sop_gb300_shim.cu) against the headers of
# a samchogroup/SOP source tree: $1, else $SOP_REFERENCE_DIR, else
# /root/reference.  Exit 3 when no such tree is present; the object goes to
# a temporary directory and is deleted.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(cd "$here/../.." && pwd)"
ref="${1:-${SOP_REFERENCE_DIR:-/root/reference}}"
if [ ! -f "$ref/global.h" ]; then
  echo "check_shim: no reference tree at $ref" >&2
  exit 3
fi
tmp="$(mktemp -d)"
trap 'rm -rf "$tmp"' EXIT
"${NVCC:-nvcc}" -std=c++14 -w -gencode arch=compute_103a,code=sm_103a \
  -I "$ref" -I "$root/oracle/stubs" -I "$root/include" \
  -c "$here/sop_gb300_shim.cu" -o "$tmp/shim.o"
echo "check_shim: compiled against $ref"
