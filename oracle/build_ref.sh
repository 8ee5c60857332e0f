#!/bin/sh
# Builds the reference's own CPU path from its sources, for cross-checking the
# oracle (test infrastructure only). Reads the reference checkout at $1
# (default /root/reference), compiles its few C files directly with gcc (not
# its build system) and writes only into oracle/_ref/:
#   sgm_ref_d{64,128,256}_p{4,8}  common/sgm_ref.c + harness.c + util.c (Makefile:40-41 flags)
#   sgm_ms_ref                    multiscale/sgm_ms_ref.c + util.c (OpenMP)
#   gen_synthetic_d{64,128,256}   common/gen_synthetic.c
#   sgm_gb300_harness_d64_p4      the reference's harness.c + util.c linked against this
#                                 engine's sgm.h plugin (when it is built): the drop-in link
set -eu
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/common/sgm_ref.c" ] || { echo "no reference checkout at $REF" >&2; exit 1; }
mkdir -p "$OUT"
CFLAGS="-O2 -Wall -Wextra -std=gnu11 -I$REF/common"
for D in 64 128 256; do
  for P in 4 8; do
    gcc $CFLAGS -DSGM_D=$D -DSGM_PATHS=$P -DGIT_SHA='"ref"' -DCFLAGS_STR='"-O2"' \
        -o "$OUT/sgm_ref_d${D}_p${P}" "$REF/common/sgm_ref.c" "$REF/common/harness.c" "$REF/common/util.c" -lm
  done
  gcc -O2 -Wall -I"$REF/common" -DSGM_D=$D -o "$OUT/gen_synthetic_d$D" "$REF/common/gen_synthetic.c" -lm
done
gcc -O2 -Wall -std=gnu11 -fopenmp -I"$REF/common" -o "$OUT/sgm_ms_ref" "$REF/multiscale/sgm_ms_ref.c" "$REF/common/util.c" -lm
PLUG="$HERE/../sgm-bench_gb300/_build"
if [ -f "$PLUG/libsgm_gb300_d64_p4.so" ]; then
  gcc $CFLAGS -DGIT_SHA='"gb300"' -DCFLAGS_STR='"gb300 sm_103a"' -o "$OUT/sgm_gb300_harness_d64_p4" \
      "$REF/common/harness.c" "$REF/common/util.c" -L"$PLUG" -lsgm_gb300_d64_p4 -Wl,-rpath,"$PLUG" -lm
fi
echo "$OUT"
