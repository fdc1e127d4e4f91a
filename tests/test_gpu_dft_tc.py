"""GPU: the blocked FP32 DFT contraction on the tensor cores (tcgen05,
3xTF32) against the same contraction on the CUDA cores, and both against the
FP64 oracle, on seeded random problems (partial blocks, several blocks)."""
import os

import numpy as np
import pytest

from harness import random_problem, relerr
from meep_gb300 import _lib

pytestmark = pytest.mark.gpu


def _run(lib, seed, dim, prec, cuda_cores, steps):
    old = os.environ.pop("MFD_DFT_CUDA_CORES", None)
    if cuda_cores:
        os.environ["MFD_DFT_CUDA_CORES"] = "1"
    try:
        eng = _lib.Engine(lib)
        return random_problem(lambda **k: _lib.Sim(eng, **k), seed, dim, precision=prec, steps=steps)
    finally:
        os.environ.pop("MFD_DFT_CUDA_CORES", None)
        if old is not None:
            os.environ["MFD_DFT_CUDA_CORES"] = old


@pytest.mark.parametrize("dim,steps", [(2, 60), (3, 60), (2, 400)])
def test_tensor_core_dft_matches_cuda_cores(dim, steps, engine_lib, oracle_lib):
    tc = _run(engine_lib, 21, dim, 32, False, steps)
    cc = _run(engine_lib, 21, dim, 32, True, steps)
    ref = _run(oracle_lib, 21, dim, 64, False, steps)
    for k in ref:
        if k.startswith("dft") or k == "flux":
            a = np.asarray(tc[k]).reshape(-1)
            b = np.asarray(cc[k]).reshape(-1)
            r = np.asarray(ref[k]).reshape(-1)
            split = lambda z: np.concatenate([np.real(z), np.imag(z)])
            assert relerr(split(a), split(b)) <= 1e-5, (k, relerr(split(a), split(b)))
            # no worse than the CUDA-core contraction against FP64
            assert relerr(split(a), split(r)) <= 2 * relerr(split(b), split(r)) + 1e-6, k
