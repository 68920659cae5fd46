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
#   tests/dropin/nbs_app.c, env_ref.c          the drop-in test application
# The shipped binaries under lib/ and bin/ are never read or linked.
#
# usage: oracle/build_ref.sh [reference dir]
#        (default $PAMR_REFERENCE_DIR, else a "reference" directory beside the repository)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${PAMR_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}}"
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

# The drop-in test application (tests/dropin/nbs_app.c) over the reference's
# own PAMR/AMRD: with amrd/mg.c (the golden run), and -- when
# libamrd_mg_gb300 is built -- with the drop-in archive in place of
# amrd/mg.o, which checks that it provides every symbol the rest of AMRD
# takes from mg.c (the link alone; running it needs a GPU).
ROOT="$(cd "$HERE/.." && pwd)"
DROP="$ROOT/tests/dropin"
APPFLAGS="$COMMON -std=gnu11 -Wall -Wno-unused-function -Wno-comment -I$DROP -I$ROOT/pamr_amrd_gb300/csrc -I$ROOT/include"
$CC $APPFLAGS -c "$DROP/env_ref.c" -o "$OUT/obj/app_env_ref.o" &
$CC $APPFLAGS -c "$DROP/nbs_app.c" -o "$OUT/obj/app_nbs.o" &
$CC $APPFLAGS -DDEVICE_MG -c "$DROP/nbs_app.c" -o "$OUT/obj/app_nbs_dev.o" &
wait
ref_objs=()
for o in "${objs[@]}"; do
  case "$o" in *own_ref_main.o) ;; *) ref_objs+=("$o") ;; esac
done
$CC -o "$OUT/nbs_app_ref" "$OUT/obj/app_nbs.o" "$OUT/obj/app_env_ref.o" "${ref_objs[@]}" -lm
echo "build_ref: $OUT/nbs_app_ref"
PKG="$ROOT/pamr_amrd_gb300"
if [ -f "$PKG/libamrd_mg_gb300.a" ] && [ -f "$PKG/libpamr_gb300.so" ]; then
  no_mg=()
  for o in "${ref_objs[@]}"; do
    case "$o" in *ref_amrd_mg.o) ;; *) no_mg+=("$o") ;; esac
  done
  CUDA_LIB="${CUDA_HOME:-/usr/local/cuda}/lib64"
  $CC -o "$OUT/nbs_app_dropin_linked" "$OUT/obj/app_nbs_dev.o" "$OUT/obj/app_env_ref.o" "${no_mg[@]}" \
      "$PKG/libamrd_mg_gb300.a" -L"$PKG" -lpamr_gb300 -L"$CUDA_LIB" -lcudart -lm \
      -Wl,-rpath,"$PKG" -Wl,-rpath,"$CUDA_LIB"
  echo "build_ref: $OUT/nbs_app_dropin_linked"
fi
