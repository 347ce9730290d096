"""Config 1 (lamellar 32^3, f=0.5, chiN=20, box 4.0, Ns=100, FP64, simple
mixing lambda=0.1, run to |dw| < 1e-8) through the C ABI on the GPU, against
the oracle's converged solution in tests/golden/config1_lamellar32.npz:
the first 20 residual norms, the iteration count, F and its parts, Q and phi
at 4096 seeded points."""
import numpy as np
import pytest

from test_config1_cpu import GOLDEN, config1_start

pytestmark = pytest.mark.gpu


def test_config1_converges_to_the_oracle_solution(pkg):
    g = np.load(GOLDEN)
    wa, wb = config1_start()
    with pkg.Context(nx=32, ny=32, nz=32, lx=4.0, ly=4.0, lz=4.0, hAB=20.0, fA=0.5, ds0=0.01,
                     precision=pkg.PREC_FP64, mixing=pkg.MIX_SIMPLE, wopt=0.1) as ctx:
        ctx.set_w(wa, wb)
        errs = []
        for _ in range(20):
            ctx.iterate(1)
            errs.append(ctx.residual()[0][0])
        np.testing.assert_allclose(errs, g["errs_first"], rtol=1e-9)
        it, fe = ctx.converge(1e-8, 5000)
        iters = 20 + it
        assert ctx.residual()[0][0] < 1e-8
        pha, phb, Q = ctx.pha.reshape(-1), ctx.phb.reshape(-1), ctx.Q()
    assert abs(iters - int(g["iterations"])) <= 2, (iters, int(g["iterations"]))
    assert abs(fe[0, 0] - g["F"][0]) < 1e-10
    np.testing.assert_allclose(fe[0, 1:4], g["F"][1:4], rtol=1e-9, atol=1e-10)
    assert abs(Q[0] / g["Q"][0] - 1) < 1e-10
    idx = g["sample_index"]
    np.testing.assert_allclose(pha[idx], g["pha_samples"], rtol=1e-8)
    np.testing.assert_allclose(phb[idx], g["phb_samples"], rtol=1e-8)
