"""Generate the golden fixtures of tests/test_golden.py.

They pin the oracle (the CPU restatement of the reference) against
regressions and give the GPU tests reference outputs that need no oracle
build: the 12x10x12 supercell case with one PD scalar after 1 and 3 large
steps (FP32 and FP64 restatements), and the reference's top-hat advection
fixture (module_advect_em.F:10564-10871) with and without the PD limiter.

    python tests/golden/make_golden.py      # rewrites tests/golden/*.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from wrf_gb300 import abi, cases  # noqa: E402
from _harness import OracleDomain, tophat_feeder  # noqa: E402

FIELDS = ["u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al"]


def golden_case():
    return cases.small_case(nx=12, ny=10, kde=12, n_scalar=1, seed=7)


def main():
    case = golden_case()
    out = {}
    for prec in ("f32", "f64"):
        od = OracleDomain(case, prec)
        done = 0
        for n in (1, 3):
            od.step(n - done)
            done = n
            for nm in FIELDS:
                out["%s_%d_%s" % (prec, n, nm)] = od.get(abi.FIELD_ID[nm]).astype(np.float64)
            for s in range(case.desc.n_moist + case.desc.n_scalar):
                out["%s_%d_q%d" % (prec, n, s)] = od.get(abi.species_id(s)).astype(np.float64)
    np.savez_compressed(os.path.join(HERE, "supercell_12x10x12.npz"), **out)
    feed = {"pd": tophat_feeder(1, nloops=400, every=200, precision="f64"),
            "orig": tophat_feeder(0, nloops=400, every=200, precision="f64")}
    np.savez_compressed(os.path.join(HERE, "tophat_feeder.npz"), **feed)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
