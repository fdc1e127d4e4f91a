"""Per-frequency single-precision error of the reference's own FP32 build on
the 96^3 dispersive case (golden_driver case disp3d_cube, 3000 steps, the
200-frequency DFT of Ez on a full plane): runs the reference core built by
oracle/ref/Makefile in both precisions with GOLDEN_DFT_DUMP, compares every
point's spectrum, and writes disp3d_cube_fp32_err.json beside this script
(also the fixtures disp3d_cube.f64.bin / .f32.bin).  Needs the reference
core (MEEP_REFERENCE set when building it); run in the build container.

    python tests/golden/make_fp32_error.py
"""
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
NF = 200


def per_frequency(a, b):
    d = np.abs(a - b).max(axis=0)
    m = np.abs(b).max(axis=0)
    return d / m, d / m.max(), m


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-j8"], check=True,
                   stdout=subprocess.DEVNULL)
    spectra = {}
    with tempfile.TemporaryDirectory() as tmp:
        for bits in (64, 32):
            exe = os.path.join(ROOT, "oracle", "_ref", "fp%d" % bits, "golden_driver")
            dump = os.path.join(tmp, "dft%d.bin" % bits)
            env = dict(os.environ, GOLDEN_DFT_DUMP=dump, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "8"))
            subprocess.run([exe, "disp3d_cube", os.path.join(HERE, "disp3d_cube.f%d.bin" % bits)], check=True,
                           env=env)
            spectra[bits] = np.fromfile(dump, dtype=np.complex128).reshape(-1, NF)
    per_f, glob, m = per_frequency(spectra[32], spectra[64])
    out = {"case": "disp3d_cube", "steps": 3000, "points": int(spectra[64].shape[0]), "nfreq": NF,
           "reference_fp32_vs_fp64_per_frequency": [float(x) for x in per_f],
           "reference_fp32_vs_fp64_global": [float(x) for x in glob],
           "fp64_max_per_frequency": [float(x) for x in m]}
    with open(os.path.join(HERE, "disp3d_cube_fp32_err.json"), "w") as fp:
        json.dump(out, fp)
    print("reference FP32 vs FP64: max %.3g, median %.3g per frequency" % (per_f.max(), np.median(per_f)))


if __name__ == "__main__":
    main()
