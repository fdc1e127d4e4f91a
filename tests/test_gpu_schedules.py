"""GPU: the 3-D step without poles or current sources, its integrated
sources away from the E slabs, runs as one CUDA graph (its source values set
on the graph's nodes each step): against the oracle, FP64 bit for bit, with
one source of four points (nsrc=1) and with three (nsrc=3)."""
import pytest

from harness import random_problem, relerr
from meep_gb300 import _lib

pytestmark = pytest.mark.gpu


def _run(lib, seed, prec, **kw):
    eng = _lib.Engine(lib)
    return random_problem(lambda **k: _lib.Sim(eng, **k), seed, 3, precision=prec, **kw)


# sources in the interior: away from every PML slab (up to 6 cells)
GRAPH = dict(n=(20, 18, 40), poles=False, ecur=False, hcur=False, src_box=((7, 7, 12), (12, 10, 28)), steps=60)


# decimation 1: an E sample after every step, each waited for before the
# next step's graph starts
@pytest.mark.parametrize("nsrc,dec", [(3, 2), (1, 2), (3, 1)])
def test_graph_step_fp64_bitwise(nsrc, dec, engine_lib, oracle_lib):
    g = _run(engine_lib, 81, 64, nsrc=nsrc, decimation=dec, **GRAPH)
    o = _run(oracle_lib, 81, 64, nsrc=nsrc, decimation=dec, **GRAPH)
    for k in o:
        assert relerr(g[k], o[k]) <= 1e-12, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("nsrc,dec", [(3, 2), (1, 2), (3, 1)])
def test_graph_step_fp32(nsrc, dec, engine_lib, oracle_lib):
    g = _run(engine_lib, 82, 32, nsrc=nsrc, decimation=dec, **GRAPH)
    o = _run(oracle_lib, 82, 32, nsrc=nsrc, decimation=dec, **GRAPH)
    for k in o:
        assert relerr(g[k], o[k]) <= 2e-5, (k, relerr(g[k], o[k]))
