#!/bin/sh
# Builds the reference's own CPU path from its sources (test infrastructure
# only): the cross-check of the oracle and the timed reference CPU baseline.
#
# Where the sources come from: the reference checkout named by $1 or by
# $SGM_REFERENCE_DIR (this recipe's default is the checkout location of the
# build container). Its few C files are staged, unchanged, into oracle/_ref/src/
# (git-ignored: never committed), so that a machine without the checkout -- an
# Arm GPU host, where the x86 binaries built here do not run -- rebuilds them
# from that copy. Without the checkout the staged copy is used; with neither,
# the recipe prints a note and builds nothing (exit 0).
#
# It compiles those files directly with gcc (not the reference's own build
# system) and writes only into oracle/_ref/:
#   sgm_ref_d{64,128,256}_p{4,8}    common/sgm_ref.c + harness.c + util.c (Makefile:40-41 flags)
#   libsgm_ref_d{64,128}_p{4,8}.so  common/sgm_ref.c + util.c as a shared library exporting the
#                                   reference's SGM_IMPL (common/sgm.h:27-40), for in-process calls
#   sgm_ms_ref                      multiscale/sgm_ms_ref.c + util.c (OpenMP)
#   gen_synthetic_d{64,128,256}     common/gen_synthetic.c
#   sgm_gb300_harness_d64_p4        the reference's harness.c + util.c linked against this
#                                   engine's sgm.h plugin (when it is built): the drop-in link
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$OUT/src"
REF=${1:-${SGM_REFERENCE_DIR:-/root/reference}}
FILES="common/sgm_ref.c common/sgm.h common/sgm_params.h common/util.c common/harness.c common/roofline.h
common/gen_synthetic.c multiscale/sgm_ms_ref.c"
if [ -f "$REF/common/sgm_ref.c" ]; then
  mkdir -p "$SRC/common" "$SRC/multiscale"
  for f in $FILES; do cp "$REF/$f" "$SRC/$f"; done
elif [ ! -f "$SRC/common/sgm_ref.c" ]; then
  echo "build_ref.sh: no reference sources (checkout or staged copy); nothing built" >&2
  exit 0
fi
C="$SRC/common"
CFLAGS="-O2 -Wall -Wextra -std=gnu11 -I$C"
OMP=-fopenmp
echo 'int main(void){return 0;}' > "$OUT/.omp_probe.c"
gcc -fopenmp "$OUT/.omp_probe.c" -o "$OUT/.omp_probe" 2>/dev/null || OMP=""
rm -f "$OUT/.omp_probe.c" "$OUT/.omp_probe"

# every compile runs in the background; each one's status is checked at the end
PIDS=""
job() { "$@" & PIDS="$PIDS $!"; }
for D in 64 128 256; do
  for P in 4 8; do
    job gcc $CFLAGS -DSGM_D=$D -DSGM_PATHS=$P -DGIT_SHA='"ref"' -DCFLAGS_STR='"-O2"' \
        -o "$OUT/sgm_ref_d${D}_p${P}" "$C/sgm_ref.c" "$C/harness.c" "$C/util.c" -lm
  done
  job gcc -O2 -Wall -I"$C" -DSGM_D=$D -o "$OUT/gen_synthetic_d$D" "$C/gen_synthetic.c" -lm
done
for D in 64 128; do
  for P in 4 8; do
    job gcc $CFLAGS -fPIC -shared -DSGM_D=$D -DSGM_PATHS=$P -o "$OUT/libsgm_ref_d${D}_p${P}.so" \
        "$C/sgm_ref.c" "$C/util.c" -lm
  done
done
job gcc -O2 -Wall -std=gnu11 $OMP -I"$C" -o "$OUT/sgm_ms_ref" "$SRC/multiscale/sgm_ms_ref.c" "$C/util.c" -lm
PLUG="$HERE/../sgm-bench_gb300/_build"
if [ -f "$PLUG/libsgm_gb300_d64_p4.so" ]; then
  job gcc $CFLAGS -DGIT_SHA='"gb300"' -DCFLAGS_STR='"gb300 sm_103a"' -o "$OUT/sgm_gb300_harness_d64_p4" \
      "$C/harness.c" "$C/util.c" -L"$PLUG" -lsgm_gb300_d64_p4 -Wl,-rpath,"$PLUG" -lm
fi
FAIL=0
for p in $PIDS; do wait "$p" || FAIL=1; done
[ "$FAIL" -eq 0 ] || { echo "build_ref.sh: a compile step failed" >&2; exit 1; }
# which OpenMP the multi-scale reference was built with, for the timing record
if [ -n "$OMP" ]; then echo openmp > "$OUT/sgm_ms_ref.omp"; else echo none > "$OUT/sgm_ms_ref.omp"; fi
echo "$OUT"
