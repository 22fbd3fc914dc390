#!/bin/sh
# Compiles the reference's hot-path C sources, where they lie, together with
# the link stubs and the harness into oracle/_ref/libvpref.so (TEST
# INFRASTRUCTURE ONLY; nothing is copied out of the reference tree).
# Exit status 2 means the reference tree is not present on this machine.
set -e
REF=${VP_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
# `build_ref.sh --root` prints where the reference tree is looked for
# (VP_REFERENCE, else the checkout this recipe was written against)
if [ "$1" = "--root" ]; then
	echo "$REF"
	exit 0
fi
OUT="$HERE/_ref"
if [ ! -f "$REF/src/chunkset/mesher.c" ]; then
	echo "reference sources not found under $REF" >&2
	exit 2
fi
mkdir -p "$OUT"
gcc -O2 -std=gnu99 -fcommon -fopenmp -w -fPIC -shared -ffp-contract=off \
	-Wl,-Bsymbolic -I"$HERE/refshim" -I"$REF/src" \
	-o "$OUT/libvpref.so" \
	"$REF/src/chunkset.c" "$REF/src/chunkset/rle.c" \
	"$REF/src/chunkset/mesher.c" "$REF/src/chunkset/edit.c" "$REF/src/gfx/fcull.c" \
	"$HERE/refshim/ref_stubs.c" "$HERE/ref_harness.c" -lm
echo "built $OUT/libvpref.so"
