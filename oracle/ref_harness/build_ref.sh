#!/usr/bin/env bash
# Builds the reference-side test harnesses from the read-only reference tree,
# in place, with outputs only under oracle/_ref/. Needs the reference checkout:
# RISA_REF_ROOT if set, else the path in oracle/ref_harness/reference_root (the
# one place that names it); prints where it looked and exits 0 without it.
#   librisa_ref_host.so : the reference's host-side table builders (CPU only)
#   risa_*.cubin        : the reference's stage kernels for sm_103a (device code
#                         only; they travel to the GPU host, where
#                         build_launch.sh builds the launcher that runs them)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${RISA_REF_ROOT:-$(head -n1 "$HERE/reference_root")}"
OUT="$HERE/../_ref"
if [ ! -d "$REF/RISA/risaLib/src" ]; then
  echo "build_ref: no reference tree at '$REF' (set RISA_REF_ROOT or edit oracle/ref_harness/reference_root); skipping"; exit 0
fi
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
INC=(-I"$HERE" -I"$HERE/stubs" -I"$REF/RISA/risaLib/src" -I"$REF/RISA/risaLib/include"
     -I"$REF/RISA/glados/include")
FLAGS=(-std=c++17 -O2 -Xcompiler -fPIC -Xcompiler -ffp-contract=off
       -include "$HERE/stubs/risa_ref_preinclude.h" -w -diag-suppress 20012,550,177)
pids=()
for tu in ref_host_fan2para ref_host_attenuation ref_host_filter; do
  "$NVCC" "${FLAGS[@]}" "${INC[@]}" -c "$HERE/$tu.cu" -o "$OUT/$tu.o" & pids+=($!)
done
# The stages' readConfig paths reference ConfigReader's constructor.
"$NVCC" "${FLAGS[@]}" "${INC[@]}" -x cu -c "$REF/RISA/risaLib/src/ConfigReader/ConfigReader.cpp" \
  -o "$OUT/ref_host_configreader.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -shared -o "$OUT/librisa_ref_host.so" "$OUT"/ref_host_*.o -lcufft -lgomp
echo "build_ref: wrote $OUT/librisa_ref_host.so"
# The reference's own stage kernels as device-only sm_103a cubins, compiled
# in place from the stage sources with the reference's nvcc flags
# (-O3 -use_fast_math); ref_launch.c loads and launches them on the GPU host.
pids=()
for stage in Attenuation Fan2Para Filter Backprojection Masking Reordering; do
  lc="$(echo "$stage" | tr '[:upper:]' '[:lower:]')"
  printf '#include "std_preinclude.h"\n#include "%s/%s.cu"\n' "$stage" "$stage" > "$OUT/risa_$lc.cu"
  "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -use_fast_math -std=c++17 "${INC[@]}" \
    -include "$HERE/stubs/risa_ref_preinclude.h" -w -o "$OUT/risa_$lc.cubin" "$OUT/risa_$lc.cu" & pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
echo "build_ref: wrote $OUT/risa_*.cubin"
