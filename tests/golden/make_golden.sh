#!/bin/sh
# Regenerates the golden fixtures in this directory from the reference core
# built by oracle/ref/Makefile (needs the reference sources; run in the build
# container, not on the GPU host).  Each case is written twice: by the FP64
# (.f64.bin) and by the FP32 (.f32.bin) reference build.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
make -C "$ROOT/oracle/ref" -j8 >/dev/null
CASES=${CASES:-"known tm2d_small tm2d_small_dec1 vec3d_small disp3d_small tm2d_full"}
for c in $CASES; do
  for p in f64 f32; do
    OMP_NUM_THREADS=${OMP_NUM_THREADS:-8} "$ROOT/oracle/_ref/fp${p#f}/golden_driver" "$c" "$HERE/$c.$p.bin"
  done
done
