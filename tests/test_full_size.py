"""Bitwise parity at the full 512 x 512 x 80 size of the throughput workload
(qv and 10 positive-definite scalars, 16 x 64 tiles of 32 x 8), periodic and
open on all four sides: one large step on the GPU against the FP32 oracle
(OpenMP over j-tiles, whose results do not depend on the tiling), every
state field and all 11 species, current and old, bit for bit.

The state takes about 7.5 GB on the device and a few times that on the
host; the oracle's step takes seconds on the host's cores.
"""
import os

import pytest

from wrf_gb300 import cases
from wrf_gb300 import gpu as G

from _harness import OracleDomain
from test_gpu_parity import _bitwise_diffs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    return cases.config2()


def _one_step_bitwise(case):
    od = OracleDomain(case, "f32", nthreads=os.cpu_count() or 1)
    od.step(1)
    ge = G.Domain(case)
    ge.step(1)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od)
    del ge, od
    return bad


def test_c2_512x512x80_one_step_bitwise(gpulib, c2):
    bad = _one_step_bitwise(c2)
    assert not bad, "\n".join(bad)


def test_c2_512x512x80_open_one_step_bitwise(gpulib, c2):
    bad = _one_step_bitwise(cases.open_boundaries(c2))
    assert not bad, "\n".join(bad)
