#!/usr/bin/env bash
# Builds the reference NuSiF sources, where they lie, into oracle/_ref/ --
# test infrastructure only (the checker and the CPU baseline), never the product.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]
#       (default: $NUSIF_REFERENCE, else /root/reference; with NUSIF_REF_OPTIONAL=1
#        a missing source tree exits 0 without building)
#
# Outputs (git-ignored; nothing is written into the reference tree):
#   _ref/libnusif_ref_rb.so   reference objects + oracle/ref_driver.c, SOLVER=rb
#   _ref/libnusif_ref_mg.so   the same with SOLVER=mg
#   _ref/NusifSolver-rb, _ref/NusifSolver-mg   the reference program itself
#   _ref/source_root.txt      the reference root the sources were read from
#
# Flags follow the reference's sequential GCC build (config.mk, mk/include_GCC.mk:
# -O3 -ffast-math -std=c99 -D_GNU_SOURCE -DARRAY_ALIGNMENT=64 -DVERBOSE), minus
# -DPROFILING, whose sequential build crashes at exit (src/profiler.c:104-108).
# The libraries are built twice: "strict" (-O2, no fast-math, no FMA contraction)
# pins the oracle bit-for-bit; "fast" keeps the reference's own flags for timing.
set -euo pipefail
REF="${1:-${NUSIF_REFERENCE:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$REF/src"
if [ ! -f "$SRC/solver-rb.c" ]; then
  # NUSIF_REF_OPTIONAL=1: a machine without the sources (the GPU machine) is not an error
  if [ "${NUSIF_REF_OPTIONAL:-0}" = "1" ]; then exit 0; fi
  echo "build_ref: reference sources not found under $SRC" >&2
  exit 2
fi
mkdir -p "$OUT"
CC="${CC:-gcc}"
COMMON="-std=c99 -D_GNU_SOURCE -DARRAY_ALIGNMENT=64 -DVERBOSE -U_FORTIFY_SOURCE -D_FORTIFY_SOURCE=0 -I$SRC"
FAST="-O3 -ffast-math"
STRICT="-O2 -ffp-contract=off"
LIBSRC="allocate.c comm.c discretization.c parameter.c profiler.c progress.c timing.c"

build_lib() { # $1 solver, $2 flavour-name, $3 opt flags
  local solver="$1" flav="$2" opt="$3" objs=()
  local tmp="$OUT/obj-$solver-$flav"
  mkdir -p "$tmp"
  for f in $LIBSRC solver-$solver.c; do
    "$CC" $COMMON $opt -fPIC -fvisibility=hidden -Dprintf=refdrv_printf \
      -c "$SRC/$f" -o "$tmp/${f%.c}.o"
    objs+=("$tmp/${f%.c}.o")
  done
  "$CC" $COMMON $opt -fPIC -c "$HERE/ref_driver.c" -o "$tmp/ref_driver.o"
  "$CC" -shared -o "$OUT/libnusif_ref_${solver}${flav:+_$flav}.so" "${objs[@]}" "$tmp/ref_driver.o" -lm
  rm -rf "$tmp"
}

for solver in rb mg; do
  build_lib "$solver" "" "$STRICT"
  build_lib "$solver" "fast" "$FAST"
  # the reference program itself, with its own flags
  "$CC" $COMMON $FAST -o "$OUT/NusifSolver-$solver" \
    $(for f in $LIBSRC main.c vtkWriter-seq.c solver-$solver.c; do echo "$SRC/$f"; done) -lm
done
# where the sources were found, for the tests that compile reference files
# themselves (layout probe, link test)
(cd "$REF" && pwd) > "$OUT/source_root.txt"
echo "build_ref: wrote $(ls "$OUT" | tr '\n' ' ')"
