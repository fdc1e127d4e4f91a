#!/bin/sh
# Regenerates the golden fixtures in this directory from the reference core
# built by oracle/ref/Makefile (needs the reference sources: set
# MEEP_REFERENCE to the reference checkout; not on the GPU host).  Each case
# is written twice: by the FP64 (.f64.bin) and by the FP32 (.f32.bin)
# reference build.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
make -C "$ROOT/oracle/ref" -j8 >/dev/null
CASES=${CASES:-"known tm2d_small tm2d_small_dec1 vec3d_small disp3d_small tm2d_full aniso1d aniso_te2d aniso3d offdiag_te2d aniso_bloch2d py_tm2d py_disp3d py_aniso_te2d py_aniso3d n2f_tm2d n2f_te2d n2f3d n2f_periodic2d py_n2f py_force py_energy py_ldos"}
for c in $CASES; do
  for p in f64 f32; do
    OMP_NUM_THREADS=${OMP_NUM_THREADS:-8} "$ROOT/oracle/_ref/fp${p#f}/golden_driver" "$c" "$HERE/$c.$p.bin"
  done
done
# The reference's adjoint-solver gradient (FP64 only: forward, adjoint and
# finite-difference runs of a 2-D design problem; about a minute on 8 threads).
OMP_NUM_THREADS=${OMP_NUM_THREADS:-8} "$ROOT/oracle/_ref/fp64/golden_driver" adjoint_tm2d "$HERE/adjoint_tm2d.f64.bin"
# The sphere quadrature table of the reference's subpixel averaging, as the
# reference's generator prints it (oracle/_ref/gen/sphere-quad.h): rows of
# "dim index x y z weight".
python3 - "$ROOT/oracle/_ref/gen/sphere-quad.h" "$HERE/sphere_quad.txt" <<'PY'
import re, sys
txt = open(sys.argv[1]).read()
counts = [int(v) for v in re.search(r"num_sphere_quad\[3\]\s*=\s*\{([^}]*)\}", txt).group(1).split(",")]
body = txt[txt.index("sphere_quad[3]"):]
rows = re.findall(r"\{\s*([-\d.e+]+),\s*([-\d.e+]+),\s*([-\d.e+]+),\s*([-\d.e+]+)\s*\}", body)
with open(sys.argv[2], "w") as f:
    i = 0
    for d, n in enumerate(counts):
        for j in range(n):
            f.write("%d %d %s\n" % (d + 1, j, " ".join(rows[i])))
            i += 1
PY
