"""Config 1 (lamellar 32^3, f=0.5, chiN=20, Ns=100, FP64, simple mixing
lambda=0.1): the golden fixture tests/golden/config1_lamellar32.npz holds the
oracle's converged solution (tests/golden/make_config1_golden.py, about 1300
iterations).  On the CPU: the oracle still reproduces the fixture's first 20
residual norms from the same seeded start."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "config1_lamellar32.npz")


def config1_start():
    spec = importlib.util.spec_from_file_location(
        "scft_fields", os.path.join(ROOT, "scft_ver1.01_gb300", "fields.py"))
    fl = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fl)
    return fl.lamellar(32, 32, 32, 4.0, 4.0, 4.0, 20.0, seed=0)


def test_oracle_reproduces_config1_start(orc):
    g = np.load(GOLDEN)
    wa, wb = config1_start()
    p = orc.Params(nx=32, ny=32, nz=32, lx=4.0, ly=4.0, lz=4.0, hAB=20.0, fA=0.5, ds0=0.01,
                   wopt=0.1)
    *_, errs = orc.converge_loop(wa, wb, p, 1e-30, 20, mixing="simple")
    np.testing.assert_allclose(errs, g["errs_first"], rtol=1e-12)
    assert int(g["iterations"]) > 1000 and g["errs_every50"][-1] < 1e-7
