#!/bin/bash
# ref_build.sh - builds the oracle's parity pin from the reference sources where they lie.
# TEST INFRASTRUCTURE ONLY. Output goes to oracle/_ref/ (git-ignored); nothing is copied.
#   usage: oracle/ref_build.sh [reference_root]
# The reference tree is the argument, else $CSMV_REFERENCE, else a checkout named "reference"
# beside this repository. Exits 0 without building when no tree is found (the GPU machine has none).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${CSMV_REFERENCE:-$HERE/../../reference}}"
if [ ! -f "$REF/bank/csmv_sh/API.cu" ]; then
  echo "ref_build: no reference tree at $REF; skipping"
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++20 -O1 -fPIC -shared -w -pthread -I"$HERE" -I"$HERE/ref_stub" -I"$REF" \
    "$HERE/ref_glue.cpp" -o "$HERE/_ref/libcsmv_ref.so"
echo "ref_build: built $HERE/_ref/libcsmv_ref.so from $REF"
