#!/usr/bin/env bash
# Builds oracle/_ref/libtgref.so from the reference's own CPU sources
# (tg_sparse_voxel_octree.c, tg_physics.c, tg_amanatides_woo.c, tg_math.c)
# where they lie under the reference checkout, plus oracle/ref_driver.c.
#
# Test infrastructure only: the library pins the C restatements in oracle/
# against the reference.  The product never links it.
#
# tg_math.c carries MSVC integer suffixes (tg_math.c:695-696,749-750: `1ui32`)
# that gcc rejects, so a suffix-stripped copy is made in a temporary directory
# that is deleted afterwards; only the .so lands in oracle/_ref/.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: $TGX_REFERENCE_ROOT)
set -euo pipefail
REF="${1:-${TGX_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "no reference root given (argument or TGX_REFERENCE_ROOT); skipping" >&2
    exit 0
fi
SRC="$REF/tg/src"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$SRC/graphics/tg_sparse_voxel_octree.c" ]; then
    echo "reference sources not found under $SRC; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
sed -e 's/\([0-9]\)ui32\b/\1u/g' -e 's/\([0-9]\)i32\b/\1/g' "$SRC/math/tg_math.c" > "$TMP/tg_math_nosuffix.c"
CFLAGS="-std=gnu11 -O2 -fPIC -fms-extensions -ffp-contract=off -fno-fast-math -w -DNDEBUG"
INC="-I$HERE/ref_shim -I$SRC"
gcc $CFLAGS $INC -c "$SRC/graphics/tg_sparse_voxel_octree.c" -o "$TMP/svo.o"
gcc $CFLAGS $INC -c "$SRC/physics/tg_physics.c" -o "$TMP/physics.o"
gcc $CFLAGS $INC -c "$SRC/util/tg_amanatides_woo.c" -o "$TMP/aw.o"
gcc $CFLAGS $INC -c "$TMP/tg_math_nosuffix.c" -o "$TMP/math.o"
gcc $CFLAGS $INC -c "$HERE/ref_driver.c" -o "$TMP/driver.o"
gcc -shared -o "$OUT/libtgref.so" "$TMP"/*.o -lm -Wl,--allow-multiple-definition
echo "built $OUT/libtgref.so"
