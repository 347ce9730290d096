"""GPU parity of the CUDA path (through the C ABI) against the CPU oracle.

Tolerances: the FP64 plain path must match the oracle to 1e-11 relative
(rounding-level: the oracle uses pocketfft, the kernels a hand-written
Stockham FFT); the FP32-propagation path to 2e-5 relative on propagators and
phi (single-precision FFT round-off accumulated over the contour)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-11, 1: 2e-5}

GRIDS = [
    (8, 8, 8, 3.0, 3.0, 3.0),
    (16, 12, 8, 4.0, 3.0, 2.5),
    (32, 32, 32, 4.0, 4.0, 4.0),
    (48, 48, 48, 3.8, 3.8, 3.8),      # radix 3
    (24, 20, 18, 3.0, 3.3, 2.7),      # radix 3 and 5
    (16, 16, 1, 4.0, 4.0, 2.0),       # 2D, Nz=1 constant-factor quirk
    (20, 1, 10, 3.0, 1.0, 2.0),       # Ny=1
    # grids served by the register-resident FP32 kernel (k_fast.cu)
    (64, 32, 32, 3.8, 3.0, 3.0),
    (128, 64, 32, 4.2, 7.3, 2.0),
    (64, 64, 1, 4.0, 4.0, 2.0),
    (256, 64, 8, 8.0, 3.0, 2.0),      # x, y fast; z (N=8) generic
    (106, 106, 1, 21.2, 21.2, 2.0),   # the reference's out.vtk grid: radix 53, spacing 0.2
    (96, 48, 32, 4.0, 3.0, 2.5),      # 96- and 48-point register lines, flattened y/z columns
]


def make_ctx(pkg, g, prec, batch=2, **kw):
    nx, ny, nz, lx, ly, lz = g
    return pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, batch=batch, precision=prec, **kw)


def oparams(orc, g, batch=2, **kw):
    nx, ny, nz, lx, ly, lz = g
    return orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, batch=batch, **kw)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("g", GRIDS)
def test_march_parity(pkg, orc, g, prec):
    from scft_gb300 import fields
    kw = dict(hAB=18.0, fA=0.36, ds0=0.02)
    p = oparams(orc, g, **kw)
    wa, wb = fields.gyroid(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 18.0, seed=1, batch=2)
    with make_ctx(pkg, g, prec, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.set_qint(-1)
        ctx.sov_dif_fft(pkg.Q_A, pkg.FIELD_WA, ctx.NsA, +1)
        ctx.sov_dif_fft(pkg.Q_CB, pkg.FIELD_WB, ctx.dNsB, -1)
        ref_a = orc.sov_dif_fft(np.ones_like(wa), wa, p.NsA, +1, p)
        ref_cb = orc.sov_dif_fft(np.ones_like(wb), wb, p.dNsB, -1, p)
        for s in (0, 1, p.NsA // 2, p.NsA):
            assert rel(ctx.get_q(pkg.Q_A, s), ref_a[:, s]) < TOL[prec], s
        for s in (0, p.dNsB - 1, p.dNsB // 3):
            assert rel(ctx.get_q(pkg.Q_CB, s), ref_cb[:, s]) < TOL[prec], s


# Long column lines: the fused z kernels k_zz<T, 128, 8> (the benchmark grid's
# z pass, in FP32, FP64 and double-float) and k_zz<float, 256, 16> (the 256^3
# workload's z pass), compared with the oracle slice by slice.
LONG_Z = [
    ((64, 64, 128, 3.8, 3.8, 3.8), (0, 1, 2)),
    ((128, 128, 128, 3.8, 3.8, 3.8), (0, 1, 2)),
    ((64, 32, 256, 3.0, 2.0, 8.0), (1,)),
    # 256 x 256 planes: the two-CTA cluster plane kernels (segment start and
    # end planes, fused plane pairs) around k_zz<float, 32, 4>
    ((256, 256, 32, 8.0, 8.0, 2.0), (1,)),
]


@pytest.mark.parametrize("g,prec", [(g, p) for g, ps in LONG_Z for p in ps],
                         ids=[f"{g[0]}x{g[1]}x{g[2]}-{ {0: 'fp64', 1: 'fp32', 2: 'df'}[p]}"
                              for g, ps in LONG_Z for p in ps])
def test_march_parity_long_columns(pkg, orc, g, prec):
    """sovDifFft (cuda_scft.cu:435-563) with every contour slice compared."""
    from scft_gb300 import fields
    kw = dict(hAB=18.0, fA=0.36, ds0=0.02)
    p = oparams(orc, g, batch=1, **kw)
    wa, _ = fields.gyroid(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 18.0, seed=2, batch=1)
    tol = {0: 1e-11, 1: 2e-5, 2: 1e-10}[prec]
    with make_ctx(pkg, g, prec, batch=1, **kw) as ctx:
        ctx.set_w(wa, -wa)
        ctx.set_qint(-1)
        ctx.sov_dif_fft(pkg.Q_A, pkg.FIELD_WA, ctx.NsA, +1)
        sched, _ = ctx.schedule()
        ref = orc.sov_dif_fft(np.ones_like(wa), wa, p.NsA, +1, p)
        for s_ in range(p.NsA + 1):
            assert rel(ctx.get_q(pkg.Q_A, s_), ref[:, s_]) < tol, s_
    # the fused step pairs (and with them the long z kernels) ran
    assert not sched & pkg.FLAG_NO_FUSED_STEPS


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("g", GRIDS[:5] + GRIDS[7:9])
def test_get_conc_parity(pkg, orc, g, prec):
    from scft_gb300 import fields
    kw = dict(hAB=20.0, fA=0.45, ds0=0.01)
    p = oparams(orc, g, **kw)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=2, batch=2)
    ref = orc.get_conc(wa, wb, p)
    with make_ctx(pkg, g, prec, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        assert rel(ctx.pha, ref.pha) < TOL[prec]
        assert rel(ctx.phb, ref.phb) < TOL[prec]
        assert np.abs(ctx.Q() / ref.Q - 1).max() < TOL[prec]
        assert rel(ctx.wa, ref.wa) < 1e-14           # getConc's own average_value
        assert rel(ctx.get_q(pkg.Q_B, 0), ref.qb[:, 0]) < TOL[prec]
        assert rel(ctx.get_q(pkg.Q_CA, p.NsA), ref.qca[:, p.NsA]) < TOL[prec]
        assert rel(ctx.get_q(pkg.Q_CA, 0), ref.qca[:, 0]) < TOL[prec]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("g,fA,ds0", [
    (GRIDS[1], 0.45, 0.01),    # NsA 45, dNsB 55: the 3/8 rule closes both blocks
    (GRIDS[7], 0.5, 0.01),     # 50 / 50: the 1/3 rule alone
    (GRIDS[0], 0.75, 0.25),    # 3 / 1: the 3/8 rule alone, and a one-step block
    (GRIDS[8], 0.36, 0.005),   # 72 / 128 on the fused-step kernels
])
def test_simpson_contour_parity(pkg, orc, g, fA, ds0, prec):
    """SCFT_FLAG_SIMPSON: phi from Simpson-weighted contour sums (an option;
    the reference integrates with the trapezoid rule)."""
    from scft_gb300 import fields
    kw = dict(hAB=20.0, fA=fA, ds0=ds0)
    p = oparams(orc, g, simpson=True, **kw)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=2, batch=2)
    ref = orc.get_conc(wa, wb, p)
    trap = orc.get_conc(wa, wb, oparams(orc, g, **kw))
    with make_ctx(pkg, g, prec, flags=pkg.FLAG_SIMPSON, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        assert rel(ctx.pha, ref.pha) < TOL[prec]
        assert rel(ctx.phb, ref.phb) < TOL[prec]
        assert np.abs(ctx.Q() / ref.Q - 1).max() < TOL[prec]
    # the option changes phi (by far more than the FP64 tolerance), not Q
    assert rel(ref.pha, trap.pha) > 1e4 * TOL[0]
    assert np.array_equal(ref.Q, trap.Q)


def test_simpson_uniform_field_gives_the_block_fractions(pkg):
    """w = 0: q = 1, Q = 1 and phiA = ds * (sum of the A block's weights) = fA
    for either rule (the weights of a block of n steps sum to n)."""
    for flags in (0, pkg.FLAG_SIMPSON):
        with pkg.Context(nx=16, ny=16, nz=8, fA=0.35, ds0=0.05, flags=flags) as ctx:
            z = np.zeros(ctx.shape)
            ctx.set_w(z, z)
            ctx.get_conc()
            np.testing.assert_allclose(ctx.pha, 0.35, rtol=1e-13)
            np.testing.assert_allclose(ctx.phb, 0.65, rtol=1e-13)


# register-resident passes on every axis: Nx in {64, 128}, Ny and Nz in
# {1, 32, 64, 128}, Ny*Nz a multiple of 64
DF_GRIDS = [GRIDS[7], GRIDS[8], GRIDS[9], (64, 64, 64, 3.8, 3.8, 3.8), (128, 32, 64, 5.0, 3.0, 4.0),
            (32, 32, 32, 4.0, 4.0, 4.0)]   # flattened y and z columns (Nx = 32)


@pytest.mark.parametrize("g", DF_GRIDS)
def test_double_float_parity(pkg, orc, g):
    """SCFT_PREC_DF: propagation in FP32-pair arithmetic must reach FP64-level
    agreement with the FP64 oracle (the FP32 path stops near 1e-6)."""
    from scft_gb300 import fields
    kw = dict(hAB=18.0, fA=0.36, ds0=0.01)
    p = oparams(orc, g, **kw)
    wa, wb = fields.gyroid(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 18.0, seed=4, batch=2)
    ref = orc.get_conc(wa, wb, p)
    with make_ctx(pkg, g, pkg.PREC_DF, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        assert rel(ctx.pha, ref.pha) < 1e-10
        assert rel(ctx.phb, ref.phb) < 1e-10
        assert np.abs(ctx.Q() / ref.Q - 1).max() < 1e-10
        assert rel(ctx.get_q(pkg.Q_A, p.NsA), ref.qa[:, p.NsA]) < 1e-10
        assert rel(ctx.get_q(pkg.Q_CB, 0), ref.qcb[:, 0]) < 1e-10


@pytest.mark.parametrize("g,fA,ds0", [(GRIDS[7], 0.45, 0.01), (GRIDS[8], 0.36, 0.005)])
def test_double_float_simpson_parity(pkg, orc, g, fA, ds0):
    """The double-float contour sum with Simpson weights (both weight classes,
    the closing 3/8 rule for odd blocks)."""
    from scft_gb300 import fields
    kw = dict(hAB=20.0, fA=fA, ds0=ds0)
    p = oparams(orc, g, simpson=True, **kw)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=3, batch=2)
    ref = orc.get_conc(wa, wb, p)
    with make_ctx(pkg, g, pkg.PREC_DF, flags=pkg.FLAG_SIMPSON, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        assert rel(ctx.pha, ref.pha) < 1e-10
        assert rel(ctx.phb, ref.phb) < 1e-10


def test_double_float_limits(pkg):
    """Grids without register-resident passes on every axis are refused
    (status, no fallback)."""
    for n in ((48, 48, 48), (96, 32, 32), (256, 64, 64)):
        with pytest.raises(pkg.ScftError) as e:
            pkg.Context(nx=n[0], ny=n[1], nz=n[2], precision=pkg.PREC_DF)
        assert e.value.status == pkg.ERR_UNSUPPORTED
    with pkg.Context(nx=64, ny=32, nz=32, precision=pkg.PREC_DF) as ctx:
        z = np.zeros(ctx.shape)
        ctx.set_w(z, z)
        ctx.get_conc()
        np.testing.assert_allclose(ctx.pha, 0.5, rtol=1e-13)


def test_double_float_polish_matches_fp64(pkg):
    """FP32 solve, then the double-float polish: the same saddle point as the
    plain FP64 path (F, Q and phi at FP64 level once both reach 1e-8)."""
    from scft_gb300 import fields
    g = dict(nx=64, ny=32, nz=32, lx=3.8, ly=3.8, lz=3.8, hAB=18.0, fA=0.36, ds0=0.01,
             mixing=pkg.MIX_ANDERSON, anderson_history=20, anderson_start=1e9)
    wa, wb = fields.gyroid(64, 32, 32, 3.8, 3.8, 3.8, 18.0, seed=0)
    with pkg.Context(precision=pkg.PREC_FP64, **g) as c64:
        c64.set_w(wa, wb)
        _, fe64 = c64.converge(1e-8, 2000)
        pha64, Q64 = c64.pha, c64.Q()
    with pkg.Context(precision=pkg.PREC_FP32, **g) as c32, \
            pkg.Context(precision=pkg.PREC_DF, **g) as cdf:
        c32.set_w(wa, wb)
        c32.converge(3e-5, 2000)
        cdf.copy_fields_from(c32)
        it, fedf = cdf.converge(1e-8, 2000)
        assert cdf.residual()[0][0] < 1e-8
        phadf, Qdf = cdf.pha, cdf.Q()
    assert abs(fedf[0, 0] - fe64[0, 0]) < 1e-9
    assert abs(Qdf[0] / Q64[0] - 1) < 1e-8
    # up to the translational zero mode of the converged structure
    spec = lambda a: np.abs(np.fft.rfftn(a[0]))
    assert np.abs(spec(phadf) - spec(pha64)).max() < 1e-6 * spec(pha64).max()


def test_average_value_and_phi_w(pkg, orc):
    g = GRIDS[1]
    p = oparams(orc, g, hAB=15.0)
    rng = np.random.default_rng(5)
    wa, wb, pa, pb = rng.normal(0.5, 1, (4, 2) + p.shape)
    with make_ctx(pkg, g, 0, hAB=15.0) as ctx:
        ctx.set_w(wa, wb)
        ctx.average_value(pkg.FIELD_WA)
        np.testing.assert_allclose(ctx.wa, orc.average_value(wa), rtol=0, atol=1e-14)
        ctx.set_w(wa, wb)
        ctx.set_field(pkg.FIELD_PHA, pa)
        ctx.set_field(pkg.FIELD_PHB, pb)
        ctx.phi_w()
        ra, rb, _, _ = orc.phi_w(wa, wb, pa, pb, 15.0, 0.05, 0.10)
        np.testing.assert_allclose(ctx.wa, ra, rtol=1e-15, atol=1e-14)
        np.testing.assert_allclose(ctx.wb, rb, rtol=1e-15, atol=1e-14)
        # the free energy uses the device Q; evaluate a concentration first
        ctx.get_conc()
        Qd = ctx.Q()
        fe = ctx.free_energy()
        F, fab, fw, fs, inc = orc.free_energy(ctx.wa, ctx.wb, ctx.pha, ctx.phb, Qd, 15.0)
        np.testing.assert_allclose(fe[:, 0], F, rtol=1e-12)
        np.testing.assert_allclose(fe[:, 1], fab, rtol=1e-12)
        np.testing.assert_allclose(fe[:, 2], fw, rtol=1e-12)
        np.testing.assert_allclose(fe[:, 3], fs, rtol=1e-12)
        np.testing.assert_allclose(fe[:, 4], inc, rtol=1e-12)


def test_free_loop_parity_fp64(pkg, orc, capfd):
    # Free (cuda_scft.cu:140-269): 30 iterations, printed lines every 10
    g = (16, 8, 8, 4.0, 2.0, 2.0)
    kw = dict(hAB=20.0, fA=0.5, ds0=0.01)
    p = oparams(orc, g, **kw)
    from scft_gb300 import fields
    wa, wb = fields.lamellar(16, 8, 8, 4.0, 2.0, 2.0, 20.0, seed=0, batch=2)
    ref = orc.free_loop(wa, wb, p, 30)
    with make_ctx(pkg, g, 0, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.free(30, 10)
        out = capfd.readouterr().out.strip().splitlines()
        assert rel(ctx.wa, ref.wa) < 1e-11
        assert rel(ctx.wb, ref.wb) < 1e-11
        assert rel(ctx.pha, ref.pha) < 1e-11
    lines = [l for l in out if l.startswith("GPU ")]
    assert len(lines) == 6
    for l, row in zip(lines, ref.log):
        it, b, F, fab, fw, fs, inc = row
        vals = [float(v) for v in l.split(":")[2].split(",")]
        assert l.startswith("GPU 0 batch %d: %5d :" % (b, it))
        np.testing.assert_allclose(vals, [F, fab, fw, fs, inc], rtol=1e-7, atol=1e-12)


def test_iterate_matches_free(pkg, orc):
    g = (16, 8, 8, 4.0, 2.0, 2.0)
    from scft_gb300 import fields
    wa, wb = fields.lamellar(16, 8, 8, 4.0, 2.0, 2.0, 20.0, seed=0, batch=1)
    p = oparams(orc, g, batch=1, hAB=20.0)
    ref = orc.free_loop(wa, wb, p, 10)
    with make_ctx(pkg, g, 0, batch=1, hAB=20.0) as ctx:
        ctx.set_w(wa, wb)
        fe = ctx.iterate(10, with_energy=True)
    F, fab, fw, fs, inc = ref.log[-1][2:]
    np.testing.assert_allclose(fe[0], [F, fab, fw, fs, inc], rtol=1e-10)


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-6)])
def test_full_size_properties_128(pkg, prec, tol):
    # 128^3, Ns=200: size-independent identities of the discretisation
    from scft_gb300 import fields
    n, L = 128, 3.8
    with pkg.Context(nx=n, ny=n, nz=n, lx=L, ly=L, lz=L, hAB=18.0, fA=0.36, ds0=0.005,
                     precision=prec) as ctx:
        # zero field: Q == 1, phiA == NsA*ds, phiB == dNsB*ds
        z = np.zeros(ctx.shape)
        ctx.set_w(z, z)
        ctx.get_conc()
        assert abs(ctx.Q()[0] - 1) < tol
        assert np.abs(ctx.pha - ctx.NsA * 0.005).max() < tol
        # gyroid field: mean(phiA + phiB) == ds*(NsA + dNsB) (W D W is symmetric)
        wa, wb = fields.gyroid(n, n, n, L, L, L, 18.0, seed=0)
        ctx.set_w(wa, wb)
        ctx.get_conc()
        tot = (ctx.pha + ctx.phb).mean()
        assert abs(tot - 0.005 * (ctx.NsA + ctx.dNsB)) < 5 * tol
        assert np.isfinite(ctx.Q()).all()


def test_full_size_properties_256(pkg):
    # config 5 at full size (256^3, Ns=400, f=0.45, chiN=22, box 8.0, the
    # lamellar/gyroid mixture), FP32: the same identities, and Q from the
    # backward chain's last slice equal to Q from the forward chain's
    from scft_gb300 import fields
    n, L, ds = 256, 8.0, 0.0025
    with pkg.Context(nx=n, ny=n, nz=n, lx=L, ly=L, lz=L, hAB=22.0, fA=0.45, ds0=ds,
                     precision=1) as ctx:
        assert (ctx.NsA, ctx.dNsB) == (180, 220)
        z = np.zeros(ctx.shape)
        ctx.set_w(z, z)
        ctx.get_conc()
        assert abs(ctx.Q()[0] - 1) < 2e-6
        assert np.abs(ctx.pha - ctx.NsA * ds).max() < 2e-6
        wa, wb = fields.mixture(n, n, n, L, L, L, 22.0, seed=0, periods=2)
        ctx.set_w(wa, wb)
        ctx.get_conc()
        tot = (ctx.pha + ctx.phb).mean()
        assert abs(tot - ds * (ctx.NsA + ctx.dNsB)) < 1e-5
        Q = ctx.Q()[0]
        assert abs(ctx.get_q(pkg.Q_CA, 0).mean() / Q - 1) < 2e-5
        assert np.isfinite(ctx.pha).all() and np.isfinite(ctx.phb).all()


def test_full_size_fp32_vs_fp64_128(pkg):
    from scft_gb300 import fields
    n, L = 128, 3.8
    wa, wb = fields.gyroid(n, n, n, L, L, L, 18.0, seed=0)
    out = {}
    for prec in (0, 1):
        with pkg.Context(nx=n, ny=n, nz=n, lx=L, ly=L, lz=L, hAB=18.0, fA=0.36, ds0=0.005,
                         precision=prec) as ctx:
            ctx.set_w(wa, wb)
            ctx.get_conc()
            out[prec] = (ctx.pha, ctx.Q())
    assert rel(out[1][0], out[0][0]) < 1e-5
    assert abs(out[1][1][0] / out[0][1][0] - 1) < 1e-5


def test_file_io_roundtrip(pkg, tmp_path):
    g = GRIDS[1]
    rng = np.random.default_rng(0)
    with make_ctx(pkg, g, 0) as ctx:
        wa, wb = rng.normal(0, 1, (2,) + ctx.shape)
        ctx.set_w(wa, wb)
        ctx.get_conc()
        f = str(tmp_path / "pha_2.dat")
        ctx.write_pha_dat(f, 1)
        pha, wa_dev = ctx.pha, ctx.wa   # getConc mean-subtracted wa on the device
        ctx.set_w(np.zeros(ctx.shape), np.zeros(ctx.shape))
        ctx.read_phi_dat(f, 0)
        np.testing.assert_allclose(ctx.wa[0], wa_dev[1], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(ctx.pha[0], pha[1], rtol=1e-5, atol=1e-6)
        assert np.all(ctx.wa[1] == 0)


def test_error_paths(pkg):
    g = GRIDS[0]
    with make_ctx(pkg, g, 0) as ctx:
        with pytest.raises(pkg.ScftError) as e:
            ctx.sov_dif_fft(pkg.Q_A, pkg.FIELD_WA, ctx.NsA + 1, 1)
        assert e.value.status == pkg.ERR_INVALID_ARG
        with pytest.raises(pkg.ScftError):
            ctx.sov_dif_fft(pkg.Q_A, pkg.FIELD_WA, 1, 0)
        with pytest.raises(pkg.ScftError) as e:
            ctx.read_phi_dat("/nonexistent/phi_1.dat")
        assert e.value.status == pkg.ERR_IO
        # a NaN field is reported, not propagated silently
        bad = np.zeros(ctx.shape)
        bad[0, 0, 0, 0] = np.nan
        ctx.set_w(bad, bad)
        ctx.get_conc()
        with pytest.raises(pkg.ScftError) as e:
            ctx.free_energy()
        assert e.value.status == pkg.ERR_NOT_FINITE
        # the context stays usable afterwards
        ctx.set_w(np.zeros(ctx.shape), np.zeros(ctx.shape))
        ctx.get_conc()
        assert abs(ctx.Q()[0] - 1) < 1e-12


def test_field_view_is_zero_copy(pkg):
    torch = pytest.importorskip("torch")
    g = (16, 12, 8, 4.0, 3.0, 2.5)
    rng = np.random.default_rng(0)
    wa = rng.normal(0, 1, (2, 8, 12, 16))
    with make_ctx(pkg, g, 0) as ctx:
        ctx.set_field(pkg.FIELD_WA, wa)
        ctx.synchronize()
        v = ctx.field_view(pkg.FIELD_WA)
        assert v.shape == (2, 8, 12, 16) and v.dtype == torch.float64 and v.is_cuda
        assert np.array_equal(v.cpu().numpy(), wa)
        v.mul_(2.0)
        torch.cuda.synchronize()
        assert np.array_equal(ctx.wa, 2.0 * wa)


@pytest.mark.parametrize("flags", ["default", "NO_XY", "NO_FUSED_STEPS", "LOCKSTEP"])
@pytest.mark.parametrize("g", [(64, 64, 64, 3.8, 3.8, 3.8), (128, 64, 32, 4.2, 3.0, 2.0),
                               (256, 64, 32, 8.0, 3.0, 2.0)])
def test_march_schedules_match_oracle(pkg, orc, g, flags):
    """Every FP32 march schedule (fused step pairs with the x+y plane or with
    three axis passes, unfused, lockstep) against the oracle, over several
    SCF iterations (the fused order changes only FP32 rounding)."""
    from scft_gb300 import fields
    kw = dict(hAB=18.0, fA=0.36, ds0=0.02)
    p = oparams(orc, g, batch=1, **kw)
    wa, wb = fields.gyroid(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 18.0, seed=4)
    f = 0 if flags == "default" else getattr(pkg, "FLAG_" + flags)
    with make_ctx(pkg, g, 1, batch=1, flags=f, **kw) as ctx:
        ctx.set_w(wa, wb)
        ctx.get_conc()
        pha, Q = ctx.pha, ctx.Q()
        sched, _ = ctx.schedule()
    ref = orc.get_conc(wa, wb, p)
    assert rel(pha, ref.pha) < TOL[1]
    assert rel(Q, ref.Q) < TOL[1]
    if flags == "default":
        assert not sched & pkg.FLAG_NO_FUSED_STEPS
