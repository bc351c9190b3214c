#!/usr/bin/env bash
# Builds oracle/_ref/librisa_ref_launch.so from ref_launch.c on the machine it
# runs on (the launcher is host code: it must be compiled where it runs).
# Needs the cubins that build_ref.sh wrote; prints a note and exits 0 without them.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/../_ref"
if [ ! -f "$OUT/risa_backprojection.cubin" ]; then
  echo "build_launch: no reference cubins in $OUT; skipping"; exit 0
fi
CUDA="${CUDA_HOME:-/usr/local/cuda}"
gcc -O2 -fPIC -shared -I"$CUDA/include" -o "$OUT/librisa_ref_launch.so" "$HERE/ref_launch.c" \
  -L"$CUDA/lib64" -L"$CUDA/lib64/stubs" -lcuda -lcufft -Wl,-rpath,"$CUDA/lib64"
echo "build_launch: wrote $OUT/librisa_ref_launch.so"
