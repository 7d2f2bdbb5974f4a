#!/usr/bin/env bash
# Compile the reference's own CPU relation code (tlranda/TetraGPU:
# src/cpu_extraction.cpp, src/validate.cpp, src/metrics.cpp) unmodified, from
# the reference source tree, together with oracle/ref_driver.cpp, into
# oracle/_ref/libtgref.so.  TEST INFRASTRUCTURE ONLY.
#
# The reference's CPU path needs two things its CMake build would provide:
#   * vtkCellTypes.h, of which it uses only the vtkIdType typedef -- a one-line
#     shim written here (VTK itself is not needed by the CPU path);
#   * datatypes.h, configured from include/datatypes.h.in with VALIDATE_GPU
#     defined (the configure step of CMakeLists.txt:15-19).
# Everything is written under oracle/_ref/, which git ignores.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $TG_REFERENCE_ROOT, else /root/reference.
# Exits 2 when the tree is absent.  The root it used is recorded in
# oracle/_ref/reference_root for the tests that compile against its headers.
set -euo pipefail
REF="${1:-${TG_REFERENCE_ROOT:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/cpu_extraction.cpp" ]; then
    echo "build_ref.sh: reference source tree not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT/include"
cat > "$OUT/include/vtkCellTypes.h" <<'EOF'
/* stand-in for VTK's header: the CPU relation code only needs vtkIdType */
#pragma once
#include <algorithm>
#include <cstdint>
#include <iostream>
#include <map>
#include <string>
#include <vector>
typedef long long vtkIdType;
EOF
sed 's/#cmakedefine VALIDATE_GPU/#define VALIDATE_GPU/' "$REF/include/datatypes.h.in" > "$OUT/include/datatypes.h"
CXX="${CXX:-g++}"
FLAGS="-std=c++17 -O2 -fPIC -w -I$OUT/include -I$REF/include"
objs=()
for src in "$REF/src/cpu_extraction.cpp" "$REF/src/validate.cpp" "$REF/src/metrics.cpp" "$HERE/ref_driver.cpp"; do
    obj="$OUT/$(basename "${src%.cpp}").o"
    $CXX $FLAGS -c "$src" -o "$obj" &
    objs+=("$obj")
done
wait
$CXX -shared -o "$OUT/libtgref.so" "${objs[@]}"
printf '%s\n' "$(cd "$REF" && pwd)" > "$OUT/reference_root"
echo "built $OUT/libtgref.so"
