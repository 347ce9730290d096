"""Live parity of the CUDA path against the reference's own kernels + cuFFT
(oracle/_ref, built from the reference sources) on the same GPU, at the
benchmark-config grid sizes.  Skipped when the reference module was not
built (it needs the reference sources at build time)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def ref_mod():
    from oracle import ref_harness
    if not ref_harness.available():
        pytest.skip("reference kernel module (oracle/_ref) not built")
    return ref_harness


CFG = [
    # 64^3 double gyroid, f=0.36, chiN=18, box 3.8, Ns=200
    ((64, 64, 64), (3.8, 3.8, 3.8), 18.0, 0.36, 0.005, "gyroid"),
    # 128x128x64 hexagonal cylinders, f=0.3, chiN=25, Lx=4.2, Ly=Lx*sqrt(3), Lz=2.0, Ns=200
    ((128, 128, 64), (4.2, 4.2 * 3 ** 0.5, 2.0), 25.0, 0.3, 0.005, "hexagonal"),
    # 32^3 lamellar, f=0.5, chiN=20, box 4.0, Ns=100
    ((32, 32, 32), (4.0, 4.0, 4.0), 20.0, 0.5, 0.01, "lamellar"),
]


@pytest.mark.parametrize("cfg", CFG, ids=["gyroid64", "hex128x128x64", "lam32"])
@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 2e-5)])
def test_get_conc_vs_reference_kernels(pkg, ref_mod, cfg, prec, tol):
    from scft_gb300 import fields as fl
    grid, box, chiN, fA, ds0, init = cfg
    gen = getattr(fl, init)
    wa, wb = gen(*grid, *box, chiN, 3)
    r = ref_mod.RefSolver(*grid, *box, chiN, fA, ds0, 1)
    r.set_w(wa, wb)
    r.get_conc()
    ref_pha, ref_phb, ref_Q = r.get_field(2), r.get_field(3), r.Q()
    r.close()
    nx, ny, nz = grid
    lx, ly, lz = box
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=chiN, fA=fA, ds0=ds0,
                     precision=prec) as ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        assert rel(ctx.pha, ref_pha) < tol
        assert rel(ctx.phb, ref_phb) < tol
        assert abs(ctx.Q()[0] / ref_Q[0] - 1) < tol


def test_loop_vs_reference_kernels(pkg, ref_mod):
    from scft_gb300 import fields as fl
    grid, box, chiN, fA, ds0 = (32, 32, 32), (4.0, 4.0, 4.0), 20.0, 0.5, 0.01
    wa, wb = fl.lamellar(*grid, *box, chiN, 0)
    r = ref_mod.RefSolver(*grid, *box, chiN, fA, ds0, 1)
    r.set_w(wa, wb)
    fe_ref = r.iterate(20)
    wa_ref = r.get_field(0)
    r.close()
    with pkg.Context(nx=32, ny=32, nz=32, lx=4.0, ly=4.0, lz=4.0, hAB=chiN, fA=fA, ds0=ds0) as ctx:
        ctx.set_w(wa, wb)
        fe = ctx.iterate(20, with_energy=True)
        assert rel(ctx.wa, wa_ref) < 1e-10
    np.testing.assert_allclose(fe, fe_ref, rtol=1e-10, atol=1e-12)
