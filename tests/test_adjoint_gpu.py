"""Adjoint of getConc and the box stress on the GPU, through the C ABI.

Checks (FP64 contexts unless stated):
- stress (-d ln Q/dL from the stored propagators) against the oracle's
  spectral formula (1e-10) and central differences of the oracle's ln Q with
  h = 1e-4 L (1e-6 relative: FD truncation);
- the adjoint's vector-Jacobian product against central differences of the
  oracle's getConc functional J = <pha_bar, phiA> + <phb_bar, phiB> + Q_bar Q
  (field directions h = 1e-5, box h = 1e-4 L; 2e-6 relative);
- the exact discrete identity d ln Q / dw = -phi / M (up to getConc's mean
  subtraction of wA), to 1e-11;
- checkpoint intervals change nothing (bit-identical);
- FP32 propagation against FP64 (errors stated in the assertion bounds)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    (12, 8, 6, 3.1, 2.7, 2.2, 0.4, 0.05),
    (16, 12, 1, 3.5, 3.0, 2.0, 0.3, 0.04),     # length-1 axis (constant wave number)
    (16, 1, 10, 3.0, 1.0, 2.5, 0.5, 0.05),
]


def fields(shape, batch, seed, scale=1.5):
    rng = np.random.default_rng(seed)
    return (rng.normal(0, scale, (batch,) + shape), rng.normal(0, scale, (batch,) + shape))


def make(pkg, orc, case, batch=2, prec=0, **kw):
    nx, ny, nz, lx, ly, lz, fA, ds0 = case
    ctx = pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=15.0, fA=fA, ds0=ds0,
                      batch=batch, precision=prec, **kw)
    p = orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=15.0, fA=fA, ds0=ds0,
                   batch=batch)
    return ctx, p


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("case", CASES)
def test_stress_matches_spectral_formula_and_fd(pkg, orc, case):
    ctx, p = make(pkg, orc, case)
    with ctx:
        wa, wb = fields(p.shape, 2, 3)
        ctx.set_w(wa, wb)
        ctx.get_conc()
        sig = ctx.stress()
    assert rel(sig, orc.stress_spectral(wa, wb, p)) < 1e-10
    fd = orc.stress_fd(wa, wb, p)
    assert rel(sig, fd) < 1e-6


@pytest.mark.parametrize("case", CASES[:2])
def test_adjoint_matches_finite_differences(pkg, orc, case):
    ctx, p = make(pkg, orc, case)
    rng = np.random.default_rng(7)
    wa, wb = fields(p.shape, 2, 5)
    pbA = rng.normal(0, 1, wa.shape)
    pbB = rng.normal(0, 1, wa.shape)
    Qb = rng.normal(0, 1, 2)
    with ctx:
        ctx.set_w(wa, wb)
        gA, gB, gL = ctx.adjoint(pbA, pbB, Qb)
    J = lambda a, b, pp: orc.conc_functional(a, b, pp, pbA, pbB, Qb)
    # field directions
    for _ in range(2):
        dA = rng.normal(0, 1, wa.shape)
        dB = rng.normal(0, 1, wa.shape)
        h = 1e-5
        fd = (J(wa + h * dA, wb + h * dB, p) - J(wa - h * dA, wb - h * dB, p)) / (2 * h)
        ad = float((gA * dA).sum() + (gB * dB).sum())
        assert abs(ad - fd) < 2e-6 * max(abs(fd), 1e-3), (ad, fd)
    # box lengths (the box is shared by the batch: the sum over instances)
    lens = (p.lx, p.ly, p.lz)
    for a in range(3):
        h = 1e-4 * lens[a]
        Lp, Lm = list(lens), list(lens)
        Lp[a] += h
        Lm[a] -= h
        fd = (J(wa, wb, orc.with_box(p, *Lp)) - J(wa, wb, orc.with_box(p, *Lm))) / (2 * h)
        ad = float(gL[:, a].sum())
        assert abs(ad - fd) < 2e-6 * max(abs(fd), 1e-3), (a, ad, fd)


@pytest.mark.parametrize("fA", [0.4, 0.35])     # blocks of 8/12 and 7/13 steps
def test_adjoint_with_simpson_weights(pkg, orc, fA):
    """SCFT_FLAG_SIMPSON: the adjoint differentiates the Simpson-weighted
    contour sums (central differences of the oracle's functional)."""
    case = CASES[0][:6] + (fA, 0.05)
    ctx, p = make(pkg, orc, case, flags=pkg.FLAG_SIMPSON)
    p.simpson = True
    rng = np.random.default_rng(11)
    wa, wb = fields(p.shape, 2, 6)
    pbA = rng.normal(0, 1, wa.shape)
    pbB = rng.normal(0, 1, wa.shape)
    Qb = rng.normal(0, 1, 2)
    with ctx:
        ctx.set_w(wa, wb)
        gA, gB, gL = ctx.adjoint(pbA, pbB, Qb)
    J = lambda a, b, pp: orc.conc_functional(a, b, pp, pbA, pbB, Qb)
    dA = rng.normal(0, 1, wa.shape)
    dB = rng.normal(0, 1, wa.shape)
    h = 1e-5
    fd = (J(wa + h * dA, wb + h * dB, p) - J(wa - h * dA, wb - h * dB, p)) / (2 * h)
    ad = float((gA * dA).sum() + (gB * dB).sum())
    assert abs(ad - fd) < 2e-6 * max(abs(fd), 1e-3), (ad, fd)
    h = 1e-4 * p.lx
    fd = (J(wa, wb, orc.with_box(p, p.lx + h, p.ly, p.lz))
          - J(wa, wb, orc.with_box(p, p.lx - h, p.ly, p.lz))) / (2 * h)
    assert abs(float(gL[:, 0].sum()) - fd) < 2e-6 * max(abs(fd), 1e-3)


def test_double_float_stress_and_adjoint(pkg, orc):
    """SCFT_PREC_DF: the stress at FP64 level (the oracle's spectral formula)
    and the adjoint against central differences, on a grid with register
    kernels on every axis."""
    case = (64, 32, 32, 4.1, 3.3, 2.9, 0.4, 0.05)
    ctx, p = make(pkg, orc, case, prec=pkg.PREC_DF)
    rng = np.random.default_rng(13)
    wa, wb = fields(p.shape, 2, 8, scale=1.0)
    pbA = rng.normal(0, 1, wa.shape)
    pbB = rng.normal(0, 1, wa.shape)
    Qb = rng.normal(0, 1, 2)
    with ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        sig = ctx.stress()
        gA, gB, gL = ctx.adjoint(pbA, pbB, Qb)
    assert rel(sig, orc.stress_spectral(wa, wb, p)) < 1e-9
    J = lambda a, b, pp: orc.conc_functional(a, b, pp, pbA, pbB, Qb)
    dA = rng.normal(0, 1, wa.shape)
    dB = rng.normal(0, 1, wa.shape)
    h = 1e-5
    fd = (J(wa + h * dA, wb + h * dB, p) - J(wa - h * dA, wb - h * dB, p)) / (2 * h)
    ad = float((gA * dA).sum() + (gB * dB).sum())
    assert abs(ad - fd) < 2e-6 * max(abs(fd), 1e-3), (ad, fd)
    h = 1e-4 * p.ly
    fd = (J(wa, wb, orc.with_box(p, p.lx, p.ly + h, p.lz))
          - J(wa, wb, orc.with_box(p, p.lx, p.ly - h, p.lz))) / (2 * h)
    assert abs(float(gL[:, 1].sum()) - fd) < 2e-6 * max(abs(fd), 1e-3)


def test_dlnQ_dw_is_minus_phi_over_M(pkg, orc):
    ctx, p = make(pkg, orc, CASES[0])
    with ctx:
        wa, wb = fields(p.shape, 2, 11)
        ctx.set_w(wa, wb)
        ctx.get_conc()
        Q = ctx.Q()
        pha, phb = ctx.pha, ctx.phb
        gA, gB, gL = ctx.adjoint(Q_bar=1.0 / Q, want_L=True)
        sig = ctx.stress()
    M = p.M
    pha_mf = pha - pha.reshape(2, -1).mean(axis=1)[:, None, None, None]
    assert rel(gA, -pha_mf / M) < 1e-11
    assert rel(gB, -phb / M) < 1e-11
    # with only the ln Q seed the box part is the stress with the sign of d ln Q
    assert rel(gL, -sig) < 1e-11


def test_checkpoint_interval_changes_nothing(pkg, orc):
    ctx, p = make(pkg, orc, CASES[0], batch=1)
    rng = np.random.default_rng(2)
    with ctx:
        wa, wb = fields(p.shape, 1, 13)
        ctx.set_w(wa, wb)
        pbA, pbB = rng.normal(0, 1, wa.shape), rng.normal(0, 1, wa.shape)
        N = p.NsA + p.dNsB
        outs = [ctx.adjoint(pbA, pbB, 0.3, checkpoint_every=k) for k in (1, 3, 0, N)]
        n_default, bytes_default = ctx.adjoint_checkpoints(0)
        n_full, _ = ctx.adjoint_checkpoints(1)
    for o in outs[1:]:
        for x, y in zip(o, outs[0]):
            assert np.array_equal(x, y)
    # sqrt(N) checkpoints: O(sqrt N) slices instead of O(N)
    assert n_default <= 3 * int(np.ceil(np.sqrt(N))) + 3 < n_full
    assert bytes_default == n_default * p.M * 8


def test_adjoint_batch_is_per_instance(pkg, orc):
    case = CASES[0]
    rng = np.random.default_rng(4)
    wa, wb = fields(case[2::-1], 2, 17)
    pbA, pbB = rng.normal(0, 1, wa.shape), rng.normal(0, 1, wa.shape)
    Qb = np.array([0.4, -1.1])
    ctx, p = make(pkg, orc, case, batch=2)
    with ctx:
        ctx.set_w(wa, wb)
        both = ctx.adjoint(pbA, pbB, Qb)
    for b in range(2):
        c1, _ = make(pkg, orc, case, batch=1)
        with c1:
            c1.set_w(wa[b:b + 1], wb[b:b + 1])
            one = c1.adjoint(pbA[b:b + 1], pbB[b:b + 1], Qb[b:b + 1])
        for x, y in zip(one, both):
            assert rel(x[0], y[b]) < 1e-13


def test_fp32_adjoint_and_stress_close_to_fp64(pkg, orc):
    case = (64, 32, 32, 4.0, 3.0, 3.0, 0.36, 0.01)
    from scft_gb300 import fields as fl
    wa, wb = fl.gyroid(64, 32, 32, 4.0, 3.0, 3.0, 15.0, seed=1)
    rng = np.random.default_rng(3)
    pbA = rng.normal(0, 1, wa.shape)
    res = []
    for prec in (0, 1):
        ctx, p = make(pkg, orc, case, batch=1, prec=prec)
        with ctx:
            ctx.set_w(wa, wb)
            ctx.get_conc()
            sig = ctx.stress()
            adj = ctx.adjoint(pbA, None, 0.5)
        res.append((sig, adj))
    (s64, a64), (s32, a32) = res
    # FP32 propagation, FP64 contractions: stress to 1e-4, gradients to 1e-3
    assert rel(s32, s64) < 1e-4
    assert rel(a32[0], a64[0]) < 1e-3 and rel(a32[1], a64[1]) < 1e-3
    assert rel(a32[2], a64[2]) < 1e-3


def test_set_box_matches_fresh_context(pkg, orc):
    case = CASES[0]
    ctx, p = make(pkg, orc, case, batch=1)
    wa, wb = fields(p.shape, 1, 21)
    with ctx:
        ctx.set_w(wa, wb)
        ctx.set_box(3.4, 2.5, 2.6)
        ctx.get_conc()
        pha, Q, sig = ctx.pha, ctx.Q(), ctx.stress()
    nx, ny, nz, _, _, _, fA, ds0 = case
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=3.4, ly=2.5, lz=2.6, hAB=15.0, fA=fA, ds0=ds0) as c2:
        c2.set_w(wa, wb)
        c2.get_conc()
        assert np.array_equal(c2.pha, pha) and np.array_equal(c2.Q(), Q)
        assert np.array_equal(c2.stress(), sig)


# 1D lamellae on an Nx x 1 x 1 grid; the length-1 axes get a long box so the
# constant wave number 2 pi / L of such an axis (the reference's bin rule)
# stays a small factor
def converged_F(pkg, nx, L, seed_w, tol=1e-11):
    with pkg.Context(nx=nx, ny=1, nz=1, lx=L, ly=50.0, lz=50.0, hAB=20.0, fA=0.5, ds0=0.01,
                     mixing=pkg.MIX_ANDERSON, anderson_history=20) as c:
        c.set_w(*seed_w)
        it, fe = c.converge(tol, 20000)
        assert it < 20000
        c.get_conc()
        return fe[0, 0], c.stress()[0, 0]


def test_stress_is_derivative_of_converged_free_energy(pkg):
    """At a saddle point dF*/dL = -d ln Q/dL at fixed w (envelope theorem):
    the stress against central differences (h = 1e-4 L) of converged F."""
    from scft_gb300 import fields as fl
    nx, L = 32, 3.7
    w = fl.lamellar(nx, 1, 1, L, 50.0, 50.0, 20.0, seed=1)
    F0, sig = converged_F(pkg, nx, L, w)
    h = 1e-4 * L
    Fp, _ = converged_F(pkg, nx, L + h, w)
    Fm, _ = converged_F(pkg, nx, L - h, w)
    fd = (Fp - Fm) / (2 * h)
    assert abs(sig - fd) < 1e-4 * max(abs(fd), 1e-4), (sig, fd)


def test_relax_cell_lamellae(pkg):
    from scft_gb300 import fields as fl
    nx, L0 = 32, 3.4
    w = fl.lamellar(nx, 1, 1, L0, 50.0, 50.0, 20.0, seed=2)
    F_start, _ = converged_F(pkg, nx, L0, w)
    with pkg.Context(nx=nx, ny=1, nz=1, lx=L0, ly=50.0, lz=50.0, hAB=20.0, fA=0.5, ds0=0.01,
                     mixing=pkg.MIX_ANDERSON, anderson_history=20) as c:
        c.set_w(*w)
        rounds, sig, fe = c.relax_cell(axes_mask=1, tol_w=1e-11, tol_stress=1e-7, max_outer=40)
        L = c.box()[0]
    assert abs(sig[0]) < 1e-7 and rounds < 40
    assert fe[0] < F_start
    # the relaxed period is a stationary point of F*(L)
    Fp, _ = converged_F(pkg, nx, L * 1.01, w)
    Fm, _ = converged_F(pkg, nx, L * 0.99, w)
    assert fe[0] < Fp and fe[0] < Fm


def test_relax_cell_recovers_hexagonal_ratio(pkg):
    """Hexagonal cylinders (f=0.3, chiN=25) in the rectangular two-cylinder
    cell, started at a = 4.2 with Ly = a*sqrt(3): relaxing Lx and Ly
    independently must keep Ly/Lx = sqrt(3) (the symmetry is not imposed)
    and find a stress-free a."""
    import math
    from scft_gb300 import fields as fl
    nx, ny, nz, a0 = 64, 112, 1, 4.2
    w = fl.hexagonal(nx, ny, nz, a0, a0 * math.sqrt(3), 2.0, 25.0, seed=0)
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=a0, ly=a0 * math.sqrt(3), lz=2.0, hAB=25.0, fA=0.3,
                     ds0=0.01, mixing=pkg.MIX_ANDERSON, anderson_history=20) as c:
        c.set_w(*w)
        rounds, sig, fe = c.relax_cell(axes_mask=3, tol_w=1e-8, tol_stress=1e-6, max_outer=40,
                                       max_inner=5000)
        L = c.box()
    assert rounds < 40 and max(abs(sig[0]), abs(sig[1])) < 1e-6
    assert abs(L[1] / L[0] - math.sqrt(3)) < 1e-4
    assert 4.3 < L[0] < 4.6


def test_stress_needs_a_get_conc_at_the_current_box(pkg, orc):
    ctx, p = make(pkg, orc, CASES[0], batch=1)
    with ctx:
        with pytest.raises(pkg.ScftError):
            ctx.stress()
        ctx.set_w(*fields(p.shape, 1, 1))
        ctx.get_conc()
        ctx.stress()
        ctx.set_box(3.0, 2.0, 2.0)
        with pytest.raises(pkg.ScftError):
            ctx.stress()
