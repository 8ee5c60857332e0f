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
#   sgm_gb300_harness_d{64,128}_p4  the reference's harness.c + util.c linked against this
#                                   engine's sgm.h plugin (when it is built): the drop-in link
# and, where nvcc is present, the reference's own CUDA programs for sm_103a (Makefile:83-90 builds
# the first the same way: nvcc for the .cu, the harness and utils in C), for a same-GPU comparison:
#   sgm_cuda_opt_d{64,128}          cuda/sgm_cuda_opt.cu + harness.c + util.c (4 paths)
#   sgm_ms_cuda                     multiscale/sgm_ms_cuda.cu + util.c (its own main)
# A CUDA step that fails leaves its program out and does not fail the recipe.
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$OUT/src"
REF=${1:-${SGM_REFERENCE_DIR:-/root/reference}}
FILES="common/sgm_ref.c common/sgm.h common/sgm_params.h common/util.c common/harness.c common/roofline.h
common/gen_synthetic.c multiscale/sgm_ms_ref.c cuda/sgm_cuda_opt.cu multiscale/sgm_ms_cuda.cu"
if [ -f "$REF/common/sgm_ref.c" ]; then
  mkdir -p "$SRC/common" "$SRC/multiscale" "$SRC/cuda"
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

# every compile runs in the background, its messages into oracle/_ref/.build.log
# (the reference's sources compile with warnings); each one's status is checked at the end
PIDS=""
: > "$OUT/.build.log"
job() { "$@" 2>> "$OUT/.build.log" & PIDS="$PIDS $!"; }
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
for D in 64 128; do
  if [ -f "$PLUG/libsgm_gb300_d${D}_p4.so" ]; then
    job gcc $CFLAGS -DSGM_D=$D -DGIT_SHA='"gb300"' -DCFLAGS_STR='"gb300 sm_103a"' \
        -o "$OUT/sgm_gb300_harness_d${D}_p4" "$C/harness.c" "$C/util.c" -L"$PLUG" -lsgm_gb300_d${D}_p4 \
        -Wl,-rpath,"$PLUG" -lm
  fi
done

# the reference's CUDA programs: optional, each in its own background chain
NVCC=${NVCC:-$(command -v nvcc || true)}
[ -n "$NVCC" ] || { [ -x /usr/local/cuda/bin/nvcc ] && NVCC=/usr/local/cuda/bin/nvcc; } || true
CUPIDS=""
cujob() { name=$1; shift; ( "$@" ) > "$OUT/.$name.log" 2>&1 & CUPIDS="$CUPIDS $!:$name"; }
if [ -n "$NVCC" ] && [ -f "$SRC/cuda/sgm_cuda_opt.cu" ]; then
  ARCH="-gencode arch=compute_103a,code=sm_103a"
  for D in 64 128; do
    cujob sgm_cuda_opt_d$D sh -c "gcc $CFLAGS -DSGM_D=$D -DSGM_PATHS=4 -DGIT_SHA='\"ref\"' \
        -DCFLAGS_STR='\"nvcc -O3 sm_103a\"' -c '$C/harness.c' -o '$OUT/.harness_cu$D.o' &&
      gcc -O2 -I'$C' -c '$C/util.c' -o '$OUT/.util_cu$D.o' &&
      '$NVCC' -O3 -I'$C' $ARCH -DSGM_D=$D -DSGM_PATHS=4 -o '$OUT/sgm_cuda_opt_d$D' \
        '$SRC/cuda/sgm_cuda_opt.cu' '$OUT/.harness_cu$D.o' '$OUT/.util_cu$D.o'"
  done
  cujob sgm_ms_cuda sh -c "gcc -O2 -I'$C' -c '$C/util.c' -o '$OUT/.util_ms.o' &&
    '$NVCC' -O3 $ARCH -o '$OUT/sgm_ms_cuda' '$SRC/multiscale/sgm_ms_cuda.cu' '$OUT/.util_ms.o'"
fi
FAIL=0
for p in $PIDS; do wait "$p" || FAIL=1; done
for pn in $CUPIDS; do
  wait "${pn%%:*}" || { echo "build_ref.sh: ${pn#*:} not built (see oracle/_ref/.${pn#*:}.log)" >&2;
                        rm -f "$OUT/${pn#*:}"; }
done
[ "$FAIL" -eq 0 ] || { cat "$OUT/.build.log" >&2; echo "build_ref.sh: a compile step failed" >&2; exit 1; }
# which OpenMP the multi-scale reference was built with, for the timing record
if [ -n "$OMP" ]; then echo openmp > "$OUT/sgm_ms_ref.omp"; else echo none > "$OUT/sgm_ms_ref.omp"; fi
echo "$OUT"
