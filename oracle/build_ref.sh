#!/bin/sh
# Build the UNMODIFIED MDZ hot path into oracle/_ref/ (TEST INFRASTRUCTURE).
#
# Compiles the reference's own sources where they lie (the MDZ tree at
# MDZ_REF_ROOT, default /root/reference; sources in its src/) with the declaration-only
# headers in oracle/shim/ and links them against the system libmpfr.so.6 /
# libgmp.so.10 by full path (no -dev packages are needed).  Two variants:
#   libmdzref_d.so   long double mapped to IEEE double, no FMA contraction
#                    (-mlong-double-64 -ffp-contract=off, mpfr_get_ld ->
#                    mpfr_get_d): the reference's "double path built without
#                    FMA", the bit-exact target of the FP64 kernel.
#   libmdzref_ld.so  as shipped (x87 80-bit long double on x86-64).
# Only x86-64 has -mlong-double-64; elsewhere the script exits 0 without
# building (the oracle restatement in oracle/mdz_oracle.c covers that case).
# `build_ref.sh --root` prints the tree's location and exits (the Python
# side asks here, so this recipe is the one place that names it).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_ROOT=${MDZ_REF_ROOT:-/root/reference}
if [ "$1" = "--root" ]; then echo "$REF_ROOT"; exit 0; fi
SRC="$REF_ROOT/src"
OUT="$HERE/_ref"
if [ ! -f "$SRC/fractal.c" ]; then
    echo "build_ref: no reference sources at $SRC; skipping" >&2
    exit 0
fi
if [ "$(uname -m)" != "x86_64" ]; then
    echo "build_ref: -mlong-double-64 needs x86-64; skipping" >&2
    exit 0
fi
find_lib() {
    for d in /usr/lib/x86_64-linux-gnu /usr/lib64 /usr/lib /lib/x86_64-linux-gnu; do
        if [ -e "$d/$1" ]; then echo "$d/$1"; return 0; fi
    done
    return 1
}
MPFR=$(find_lib libmpfr.so.6) || { echo "build_ref: libmpfr.so.6 not found" >&2; exit 1; }
GMP=$(find_lib libgmp.so.10) || { echo "build_ref: libgmp.so.10 not found" >&2; exit 1; }
mkdir -p "$OUT"
FILES="frac_mandel.c frac_burning_ship.c frac_generalized_celtic.c frac_variant.c fractal.c render_threads.c coords.c my_mpfr_to_str.c timer.c debug.c"
SRCS=""
for f in $FILES; do SRCS="$SRCS $SRC/$f"; done
COMMON="-std=gnu99 -O3 -DNDEBUG -DRTH_NDEBUG -DVERSION=\"0.1.2\" -fPIC -shared -w -I$HERE/shim -I$SRC"
gcc $COMMON -mlong-double-64 -ffp-contract=off -DMDZ_SHIM_LD_AS_D \
    $SRCS "$HERE/ref_driver.c" -o "$OUT/libmdzref_d.so" "$MPFR" "$GMP" -lm -lpthread
gcc $COMMON -ffp-contract=off \
    $SRCS "$HERE/ref_driver.c" -o "$OUT/libmdzref_ld.so" "$MPFR" "$GMP" -lm -lpthread
# colouring (palette.c, render.c) and the .mdz settings loader (image_info.c,
# mdzfileio.c, setting.c) on top of the hot path, driven by ref_io_driver.c
IOFILES="palette.c render.c image_info.c mdzfileio.c setting.c globals.c cmdline.c"
IOSRCS="$SRCS"
for f in $IOFILES; do IOSRCS="$IOSRCS $SRC/$f"; done
gcc $COMMON -include limits.h -ffp-contract=off \
    $IOSRCS "$HERE/ref_io_driver.c" -o "$OUT/libmdzref_io.so" "$MPFR" "$GMP" -lm -lpthread
echo "build_ref: built $OUT/libmdzref_d.so $OUT/libmdzref_ld.so $OUT/libmdzref_io.so"
