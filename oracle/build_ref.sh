#!/usr/bin/env bash
# Builds the reference's own multigrid path (PAMR + AMRD C sources, compiled
# in place from the read-only reference tree) into oracle/_ref/ref_mg.
#
# TEST INFRASTRUCTURE (oracle only). The reference's autoconf build needs MPI,
# a Fortran compiler and RNPL's bbhutil, none of which exist here, so this
# recipe compiles the C sources directly with:
#   oracle/shim/mpi.h, oracle/shim/bbhutil.h   single-rank / parameter shims
#   oracle/m_util_r8.c                         C restatement of the Fortran kernels
#   oracle/mg_ops.c, oracle/ref_main.c         application hooks and driver
# The shipped binaries under lib/ and bin/ are never read or linked.
#
# usage: oracle/build_ref.sh [reference dir]   (default /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${PAMR_REFERENCE_DIR:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/amrd/mg.c" ]; then
  echo "build_ref: reference sources not found at $REF" >&2
  exit 1
fi
mkdir -p "$OUT/obj"
CC=${CC:-gcc}
# -ffp-contract=off: no fused multiply-add, so the arithmetic is the same on x86 and Arm
COMMON="-O2 -ffp-contract=off -fno-fast-math -fcommon -I$HERE/shim -I$REF/include -I$REF/src -I$REF/amrd -I$HERE"
objs=()
for f in src/pamr.c src/gh.c src/transfer.c src/misc.c src/io.c \
         amrd/amrd.c amrd/mg.c amrd/util.c amrd/globals.c amrd/io.c amrd/evolve.c \
         amrd/cls.c amrd/regrid_script.c; do
  o="$OUT/obj/ref_$(echo "$f" | tr '/' '_' | sed 's/\.c$/.o/')"
  $CC $COMMON -std=gnu89 -w -c "$REF/$f" -o "$o" &
  objs+=("$o")
done
for f in shim/shim.c m_util_r8.c mg_ops.c ref_main.c; do
  o="$OUT/obj/own_$(basename "$f" .c).o"
  $CC $COMMON -std=gnu11 -Wall -Wno-unused-function -Wno-comment -c "$HERE/$f" -o "$o" &
  objs+=("$o")
done
wait
$CC -o "$OUT/ref_mg" "${objs[@]}" -lm
echo "build_ref: $OUT/ref_mg"
