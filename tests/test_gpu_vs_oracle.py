"""GPU: the C ABI of the CUDA engine against the CPU oracle on the same seeded
random problems (random materials, conductivity, Drude/Lorentz poles,
integrated and current sources, DFT monitors), 2-D and 3-D, FP64 and FP32."""
import numpy as np
import pytest

from harness import random_problem, relerr
from meep_gb300 import _lib

pytestmark = pytest.mark.gpu


def _run(lib, seed, dim, prec):
    eng = _lib.Engine(lib)
    return random_problem(lambda **kw: _lib.Sim(eng, **kw), seed, dim, precision=prec)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fp64_bitwise_class(dim, seed, engine_lib, oracle_lib):
    g = _run(engine_lib, seed, dim, 64)
    o = _run(oracle_lib, seed, dim, 64)
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-12, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("dim", [2, 3])
def test_fp32_close(dim, engine_lib, oracle_lib):
    g = _run(engine_lib, 7, dim, 32)
    o = _run(oracle_lib, 7, dim, 64)
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-3, (k, relerr(g[k], o[k]))
