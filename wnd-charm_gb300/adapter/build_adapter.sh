#!/usr/bin/env bash
# Builds the reference-side adapter against the reference's own headers and
# library: gb300_executor.cpp + adapter_demo.cpp, linked with the reference
# library that oracle/build_ref.sh builds from the reference sources
# (oracle/_ref/libwndref.so) and with this project's libwndcharm_gb300.so.
# Output: wnd-charm_gb300/adapter/_build/adapter_demo.
# Usage: wnd-charm_gb300/adapter/build_adapter.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(cd "$HERE/../.." && pwd)"
if [ ! -d "$REF/src" ]; then echo "reference sources not found at $REF/src" >&2; exit 2; fi
if [ ! -f "$REPO/oracle/_ref/libwndref.so" ]; then "$REPO/oracle/build_ref.sh" "$REF" >/dev/null; fi
LIB="$REPO/wnd-charm_gb300/build"
if [ ! -f "$LIB/libwndcharm_gb300.so" ]; then echo "build libwndcharm_gb300.so first" >&2; exit 2; fi
mkdir -p "$HERE/_build"
CXX="${CXX:-g++}"
FLAGS="-O2 -std=gnu++11 -w -I$REPO/oracle/ref_shim/include -I$REF/src -I$REPO/include -I$HERE"
$CXX $FLAGS "$HERE/gb300_executor.cpp" "$HERE/adapter_demo.cpp" -o "$HERE/_build/adapter_demo" \
    -L"$REPO/oracle/_ref" -lwndref -L"$LIB" -lwndcharm_gb300 \
    -Wl,-rpath,"$REPO/oracle/_ref" -Wl,-rpath,"$LIB"
echo "built $HERE/_build/adapter_demo"
