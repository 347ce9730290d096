"""Convergence machinery on the GPU against the CPU oracle: the residual of
the field update, Anderson mixing (double-float history ring, FP64 Gram
matrix and least squares on the device), convergence to |dw| < tol, and an
FP32 solve polished in FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = (16, 16, 8, 4.0, 4.0, 2.0)


def ctx_for(pkg, prec=0, batch=2, **kw):
    nx, ny, nz, lx, ly, lz = G
    return pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=20.0, fA=0.5, ds0=0.01,
                       batch=batch, precision=prec, **kw)


def oparams(orc, batch=2):
    nx, ny, nz, lx, ly, lz = G
    return orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=20.0, fA=0.5, ds0=0.01,
                      batch=batch)


def fields(batch=2, seed=0):
    from scft_gb300 import fields as fl
    nx, ny, nz, lx, ly, lz = G
    return fl.lamellar(nx, ny, nz, lx, ly, lz, 20.0, seed=seed, batch=batch)


def test_residual_of_simple_mixing(pkg, orc):
    wa, wb = fields()
    p = oparams(orc)
    with ctx_for(pkg) as ctx:
        ctx.set_w(wa, wb)
        ctx.iterate(1)
        mx, rms = ctx.residual()
    a = orc.average_value(wa)
    b = orc.average_value(wb)
    c = orc.get_conc(a, b, p)
    _, _, emax, erms, _, _ = orc.residual(c.wa, b, c.pha, c.phb, p.hAB, p.wcmp)
    np.testing.assert_allclose(mx, emax, rtol=1e-10)
    np.testing.assert_allclose(rms, erms, rtol=1e-10)


def test_anderson_trajectory_matches_oracle(pkg, orc):
    wa, wb = fields()
    p = oparams(orc)
    kw = dict(mixing=pkg.MIX_ANDERSON, anderson_history=10, anderson_lambda=0.5,
              anderson_start=0.1)
    with ctx_for(pkg, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.iterate(60)
        ga, gb = ctx.wa, ctx.wb
    ra, rb, *_ = orc.converge_loop(wa, wb, p, 1e-30, 60, mixing="anderson", m=10, lam=0.5,
                                   start=0.1)
    scale = np.abs(ra).max()
    assert np.abs(ga - ra).max() / scale < 1e-7
    assert np.abs(gb - rb).max() / scale < 1e-7


@pytest.mark.parametrize("iters", [3, 6, 12])
def test_double_float_ring_keeps_the_fp64_trajectory(pkg, orc, iters):
    """The ring holds u = w + lambda d and d as double-float pairs (about 48
    bits) and sums them on the FP32 pipe; an FP64 context's Anderson
    trajectory (Anderson from the first step, m = 8) follows the FP64 NumPy
    restatement to 2e-9 over 12 iterations.  Measured on a GB300: 2.9e-10,
    7.1e-10, 3.7e-10 after 3, 6, 12 iterations (with an FP64 ring: 2.7e-11,
    1.3e-10, 2.3e-10).  The least-squares solve amplifies rounding in the Gram
    row, so both trajectories leave the restatement's by about 1e-5 after 30
    iterations of this start; converged results agree (tests below)."""
    wa, wb = fields(seed=1)
    p = oparams(orc)
    kw = dict(mixing=pkg.MIX_ANDERSON, anderson_history=8, anderson_lambda=0.5,
              anderson_start=10.0)
    with ctx_for(pkg, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.iterate(iters)
        ga, gb = ctx.wa, ctx.wb
    ra, rb, *_ = orc.converge_loop(wa, wb, p, 1e-30, iters, mixing="anderson", m=8, lam=0.5,
                                   start=10.0)
    scale = np.abs(ra).max()
    err = max(np.abs(ga - ra).max(), np.abs(gb - rb).max()) / scale
    assert err < 2e-9, err


def test_anderson_converges_to_oracle_saddle_point(pkg, orc):
    wa, wb = fields(batch=1, seed=3)
    p = oparams(orc, batch=1)
    kw = dict(mixing=pkg.MIX_ANDERSON, anderson_history=20, anderson_lambda=0.5,
              anderson_start=0.1)
    with ctx_for(pkg, batch=1, **kw) as ctx:
        ctx.set_w(wa, wb)
        iters, fe = ctx.converge(1e-6, 1000)
        mx, _ = ctx.residual()
        pha = ctx.pha
    assert mx[0] < 1e-6 and iters < 1000
    ra, rb, rpa, rpb, rQ, rit, errs = orc.converge_loop(wa, wb, p, 1e-6, 1000, mixing="anderson",
                                                        m=20, lam=0.5, start=0.1)
    F = orc.free_energy(ra, rb, rpa, rpb, rQ, p.hAB)[0]
    assert abs(fe[0, 0] - F[0]) < 1e-8
    assert np.abs(pha - rpa).max() < 1e-6


def test_fp32_solve_with_fp64_polish(pkg):
    wa, wb = fields(batch=1, seed=5)
    kw = dict(mixing=pkg.MIX_ANDERSON, anderson_history=20, anderson_lambda=0.5,
              anderson_start=0.1)
    with ctx_for(pkg, prec=0, batch=1, **kw) as c64:
        c64.set_w(wa, wb)
        it64, fe64 = c64.converge(1e-7, 1500)
    with ctx_for(pkg, prec=1, batch=1, **kw) as c32, ctx_for(pkg, prec=0, batch=1, **kw) as pol:
        c32.set_w(wa, wb)
        it32, _ = c32.converge(1e-4, 1500)            # FP32 residual floor is ~1e-5
        pol.copy_fields_from(c32)
        itp, fep = pol.converge(1e-7, 500)
    assert itp < it64                                  # the polish starts near the saddle point
    assert abs(fep[0, 0] - fe64[0, 0]) < 1e-7 * max(1.0, abs(fe64[0, 0]))


def test_bad_anderson_params(pkg):
    with pytest.raises(pkg.ScftError) as e:
        ctx_for(pkg, mixing=pkg.MIX_ANDERSON, anderson_history=40)
    assert e.value.status == pkg.ERR_INVALID_ARG


def test_pinned_translation_trajectory_matches_oracle(pkg, orc):
    """SCFT_FLAG_PIN_TRANSLATION: every Anderson update without its component
    along the fields' rigid shifts, against the oracle's remove_translation
    (the same least squares over both fields' central-difference gradients)."""
    wa, wb = fields()
    p = oparams(orc)
    kw = dict(mixing=pkg.MIX_ANDERSON, anderson_history=10, anderson_lambda=0.5,
              anderson_start=0.1, flags=pkg.FLAG_PIN_TRANSLATION)
    with ctx_for(pkg, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.iterate(40)
        ga, gb = ctx.wa, ctx.wb
    ra, rb, *_ = orc.converge_loop(wa, wb, p, 1e-30, 40, mixing="anderson", m=10, lam=0.5,
                                   start=0.1, pin_translation=True)
    scale = np.abs(ra).max()
    assert np.abs(ga - ra).max() / scale < 1e-7
    assert np.abs(gb - rb).max() / scale < 1e-7
    # the pinning changes the trajectory (else the test would not test it)
    ua, *_ = orc.converge_loop(wa, wb, p, 1e-30, 40, mixing="anderson", m=10, lam=0.5,
                               start=0.1)
    assert np.abs(ua - ra).max() / scale > 1e-6


def test_pinned_translation_fp32_df_polish_agrees_pointwise(pkg):
    """With the rigid shifts pinned, FP32 propagation followed by the
    double-float polish reaches the plain FP64 path's structure without any
    alignment: phi pointwise within 1e-6 relative once both reach 1e-8."""
    from scft_gb300 import fields as fl
    g = dict(nx=64, ny=32, nz=32, lx=3.8, ly=3.8, lz=3.8, hAB=18.0, fA=0.36, ds0=0.01,
             mixing=pkg.MIX_ANDERSON, anderson_history=20, anderson_start=1e9,
             flags=pkg.FLAG_PIN_TRANSLATION)
    wa, wb = fl.gyroid(64, 32, 32, 3.8, 3.8, 3.8, 18.0, seed=0)
    with pkg.Context(precision=pkg.PREC_FP64, **g) as c64:
        c64.set_w(wa, wb)
        _, fe64 = c64.converge(1e-8, 2000)
        pha64, phb64 = c64.pha, c64.phb
    with pkg.Context(precision=pkg.PREC_FP32, **g) as c32, \
            pkg.Context(precision=pkg.PREC_DF, **g) as cdf:
        c32.set_w(wa, wb)
        c32.converge(3e-5, 2000)
        cdf.copy_fields_from(c32)
        _, fedf = cdf.converge(1e-8, 2000)
        phadf, phbdf = cdf.pha, cdf.phb
    assert abs(fedf[0, 0] - fe64[0, 0]) < 1e-9
    assert np.abs(phadf - pha64).max() / np.abs(pha64).max() < 1e-6
    assert np.abs(phbdf - phb64).max() / np.abs(phb64).max() < 1e-6


def test_pin_translation_needs_anderson(pkg):
    with pytest.raises(pkg.ScftError) as e:
        ctx_for(pkg, flags=pkg.FLAG_PIN_TRANSLATION)
    assert e.value.status == pkg.ERR_INVALID_ARG
