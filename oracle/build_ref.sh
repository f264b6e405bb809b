#!/usr/bin/env bash
# Builds oracle/_ref/libsvo_ref.so: the reference's own kernel/kernel.cl,
# src/octree/octree.h and src/octree/Rle4.cpp (behind oracle/ref_win/windows.h)
# compiled for the host CPU behind oracle/ref_shim.h, one
# copy per octree depth 8..12 (OCTREE_DEPTH is hard-coded at kernel.cl:12 and
# octree.h:2, so the sources are streamed through sed into the compiler; no
# copy of them is written anywhere). TEST INFRASTRUCTURE ONLY: the library is
# the checker that pins the oracle restatement and makes the golden fixtures.
#
# usage: oracle/build_ref.sh <reference_dir>   (or SVO_REFERENCE_DIR set)
# Exits 0 without building when no reference tree is given or it is absent.
set -euo pipefail
REF="${1:-${SVO_REFERENCE_DIR:-}}"
if [ -z "$REF" ]; then
    echo "build_ref: no reference directory given (argument or SVO_REFERENCE_DIR); skipped"
    exit 0
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
KCL="$REF/kernel/kernel.cl"
OCT="$REF/src/octree/octree.h"
if [ ! -f "$KCL" ] || [ ! -f "$OCT" ]; then
    echo "build_ref: reference sources not found under $REF; skipped"
    exit 0
fi
for f in "$KCL" "$OCT"; do
    n=$(grep -c '^#define OCTREE_DEPTH 11$' "$f" || true)
    if [ "$n" != "1" ]; then echo "build_ref: expected one '#define OCTREE_DEPTH 11' in $f"; exit 1; fi
done
mkdir -p "$OUT"
{
    echo '#include "ref_shim.h"'
    for D in 8 9 10 11 12; do
        echo '#undef OCTREE_DEPTH'
        echo "namespace svo_ref_d$D {"
        echo 'namespace k {'
        echo '#line 1 "kernel/kernel.cl"'
        sed -e "s/^#define OCTREE_DEPTH 11\$/#define OCTREE_DEPTH $D/" "$KCL"
        echo '}'
        echo 'namespace b {'
        echo '#line 1 "src/octree/octree.h"'
        sed -e "s/^#define OCTREE_DEPTH 11\$/#define OCTREE_DEPTH $D/" "$OCT"
        echo '}'
        echo '#include "ref_driver.inc"'
        echo '}'
    done
    if [ -f "$REF/src/octree/Rle4.cpp" ]; then
        echo '#line 1 "src/octree/Rle4.cpp"'
        cat "$REF/src/octree/Rle4.cpp"
    fi
    echo '#include "ref_capi.inc"'
} | g++ -x c++ -std=c++17 -O2 -ffp-contract=off -fno-strict-aliasing -fPIC -shared -w \
        -I"$HERE" -I"$HERE/ref_win" -I"$REF/src/octree" -I"$REF/src" -o "$OUT/libsvo_ref.so.tmp" -
mv "$OUT/libsvo_ref.so.tmp" "$OUT/libsvo_ref.so"
echo "build_ref: built $OUT/libsvo_ref.so"
