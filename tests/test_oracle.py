"""Known-answer tests pinning the CPU oracle (no GPU).

The reference ships no tests or golden vectors for this path, so the oracle
is pinned here by exact properties of the reference's discretisation
(cuda_scft.cu:435-563, getConc :61-138) and against the reference kernels'
own outputs (tests/test_ref_golden.py)."""
import numpy as np
import pytest


def P(orc, **kw):
    base = dict(nx=16, ny=16, nz=16, lx=4.0, ly=4.0, lz=4.0, hAB=20.0, fA=0.5, ds0=0.01, batch=1)
    base.update(kw)
    return orc.Params(**base)


def test_ns_split(orc):
    # init_cuda.cu:330-331, including the 1e-8 guard against 0.36/0.005 -> 71.999
    p = P(orc, fA=0.36, ds0=0.005)
    assert (p.NsA, p.dNsB) == (72, 128)
    p = P(orc, fA=0.3, ds0=0.005)
    assert (p.NsA, p.dNsB) == (60, 140)
    p = P(orc, fA=0.45, ds0=1 / 400)
    assert (p.NsA, p.dNsB) == (180, 220)


def test_k2_axis_reference_order(orc):
    k = orc.k2_axis(8, 4.0)
    d = 4.0 / 8
    expect = [(2 * orc.PI_REF * i / 8 / d) ** 2 for i in range(4)] + \
             [(2 * orc.PI_REF * (i - 8) / d / 8) ** 2 for i in range(4, 8)]
    np.testing.assert_allclose(k, expect, rtol=1e-15)
    # length-1 axis: bin 0 takes the negative branch (i - n = -1)
    assert orc.k2_axis(1, 2.0)[0] == pytest.approx((2 * orc.PI_REF / 2.0) ** 2, rel=1e-15)


def test_zero_field_known_answer(orc):
    # w == 0: q == 1 for all s, Q == 1, phiA == NsA*ds, phiB == dNsB*ds
    p = P(orc, nx=8, ny=8, nz=8)
    z = np.zeros((1,) + p.shape)
    c = orc.get_conc(z, z, p)
    assert abs(c.Q[0] - 1) < 1e-14
    np.testing.assert_allclose(c.pha, p.NsA * p.ds0, atol=1e-14)
    np.testing.assert_allclose(c.phb, p.dNsB * p.ds0, atol=1e-14)


def test_single_mode_decays_exactly(orc):
    # w == 0: the split step is exact: a Fourier mode decays as exp(-k^2 s)
    p = P(orc, nx=16, ny=8, nz=8, lx=3.0)
    x = np.arange(p.nx) * p.lx / p.nx
    q0 = (1 + 0.3 * np.cos(2 * np.pi * 2 * x / p.lx))[None, None, None, :] * np.ones((1,) + p.shape)
    z = np.zeros((1,) + p.shape)
    q = orc.sov_dif_fft(q0, z, 20, +1, p)
    kref = 2 * orc.PI_REF * 2 / p.lx
    for s in (1, 7, 20):
        expect = 1 + 0.3 * np.exp(-kref ** 2 * p.ds0 * s) * np.cos(2 * np.pi * 2 * x / p.lx)
        np.testing.assert_allclose(q[0, s, 0, 0], expect, rtol=0, atol=1e-13)


def test_constant_field_known_answer(orc):
    # w == c: q(s) = exp(-c*s*ds)
    p = P(orc, nx=8, ny=8, nz=8)
    c = 0.7
    w = np.full((1,) + p.shape, c)
    q = orc.sov_dif_fft(np.ones_like(w), w, 10, +1, p)
    for s in range(11):
        np.testing.assert_allclose(q[0, s], np.exp(-c * s * p.ds0), rtol=1e-13)


def test_nz1_quirk_constant_factor(orc):
    # Nz=1: every mode is multiplied by exp(-ds*(2pi/lz)^2) per step
    # (init_cuda.cu:414-415 gives kz[0] = -2pi/lz); phi is unchanged, Q is scaled.
    p = P(orc, nx=16, ny=16, nz=1, lz=2.0)
    z = np.zeros((1,) + p.shape)
    c = orc.get_conc(z, z, p)
    fac = np.exp(-p.ds0 * (2 * orc.PI_REF / p.lz) ** 2)
    assert c.Q[0] == pytest.approx(fac ** (p.NsA + p.dNsB), rel=1e-12)
    np.testing.assert_allclose(c.pha + c.phb, 1.0, atol=1e-12)


def test_mass_identity(orc):
    # <q(s) q+(s)>_r is independent of s (the step operator W D W is
    # symmetric), so mean(phiA + phiB) == ds*(NsA + dNsB) for any field.
    p = P(orc, nx=12, ny=10, nz=8, fA=0.36, ds0=0.02)
    rng = np.random.default_rng(3)
    wa, wb = rng.normal(0, 2, (2, 1) + p.shape)
    c = orc.get_conc(wa, wb, p)
    assert (c.pha + c.phb).mean() == pytest.approx(p.ds0 * (p.NsA + p.dNsB), rel=1e-12)


def test_ab_swap_symmetry(orc):
    # f = 1/2: exchanging wA and wB exchanges phiA and phiB
    p = P(orc, nx=8, ny=8, nz=8, fA=0.5, ds0=0.05)
    rng = np.random.default_rng(1)
    wa, wb = rng.normal(0, 1, (2, 1) + p.shape)
    wa, wb = orc.average_value(wa), orc.average_value(wb)
    c1 = orc.get_conc(wa, wb, p)
    c2 = orc.get_conc(wb, wa, p)
    np.testing.assert_allclose(c1.pha, c2.phb, atol=1e-12)
    np.testing.assert_allclose(c1.phb, c2.pha, atol=1e-12)
    assert c1.Q[0] == pytest.approx(c2.Q[0], rel=1e-12)


def test_second_order_in_ds(orc):
    # Richardson: the split step has O(ds^2) contour error
    p0 = P(orc, nx=8, ny=8, nz=8, fA=0.5)
    x = np.arange(8) * 4.0 / 8
    smooth = np.cos(2 * np.pi * x / 4.0)[None, None, None, :] * np.ones((1,) + p0.shape)
    wa, wb = 2.0 * smooth, -2.0 * smooth
    Qs = []
    for ds in (0.02, 0.01, 0.005):
        p = P(orc, nx=8, ny=8, nz=8, fA=0.5, ds0=ds)
        Qs.append(orc.get_conc(wa, wb, p).Q[0])
    r = (Qs[0] - Qs[1]) / (Qs[1] - Qs[2])
    assert 3.5 < r < 4.5


def test_average_value(orc):
    rng = np.random.default_rng(0)
    w = rng.normal(3, 1, (3, 4, 5, 6))
    a = orc.average_value(w)
    np.testing.assert_allclose(a.reshape(3, -1).mean(axis=1), 0, atol=1e-14)


def test_simple_mixing_converges(orc):
    # the reference loop drives the incompressibility error down
    p = P(orc, nx=16, ny=4, nz=4, lx=4.0, hAB=12.0, fA=0.5, ds0=0.02)
    rng = np.random.default_rng(0)
    x = np.arange(p.nx) * p.lx / p.nx
    base = 1.2 * np.cos(2 * np.pi * x / p.lx) * np.ones(p.shape)
    wa = base[None] + rng.normal(0, 0.01, (1,) + p.shape)
    wb = -base[None] + rng.normal(0, 0.01, (1,) + p.shape)
    res = orc.free_loop(wa, wb, p, 200)
    incs = [row[6] for row in res.log]
    assert incs[-1] < incs[0]
    assert incs[-1] < 1e-2


def test_reduce3_quirk(orc):
    # reduce3 (cuda_aid.cuh:59-68) drops elements for non-power-of-two thread
    # counts, e.g. the 212 threads of a 106x106 grid; power-of-two counts are exact.
    x = np.arange(1.0, 106 * 106 + 1)
    assert orc.factor_decompose_1024(106 * 106) == 212
    assert orc.reduce3_quirk_sum(x, 212) != pytest.approx(x.sum(), rel=1e-12)
    y = np.arange(1.0, 32 ** 3 + 1)
    assert orc.factor_decompose_1024(32 ** 3) == 1024
    assert orc.reduce3_quirk_sum(y, 1024) == pytest.approx(y.sum(), rel=1e-14)


def test_pha_dat_roundtrip(orc, tmp_path):
    p = P(orc, nx=4, ny=3, nz=2)
    rng = np.random.default_rng(0)
    a, b, c, d = rng.normal(0, 1, (4, p.M))
    f = tmp_path / "pha_1.dat"
    orc.write_pha_dat(f, p, a, b, c, d)
    lines = f.read_text().splitlines()
    assert lines[0] == "Nx=4, Ny=3, Nz=2"
    assert lines[1] == "dx=%g, dy=%g, dz=%g" % (1.0, 4.0 / 3, 2.0)
    ra, rb, rc, rd = orc.read_phi_dat(f, p.M)
    np.testing.assert_allclose(ra, a, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(rd, d, rtol=1e-5, atol=1e-6)


def test_parse_ab_txt(orc):
    text = ("intag=1024\nxN=18.0\nfa=0.360\nlx=3.8, ly=3.8,  lz=3.8\n"
            "Nx=64, Ny=64, Nz=64\nds0=0.005\nbatch=2\n")
    p = orc.parse_ab_txt(text)
    assert (p.nx, p.ny, p.nz, p.batch, p.intag) == (64, 64, 64, 2, 1024)
    assert (p.hAB, p.fA, p.ds0, p.lz) == (18.0, 0.36, 0.005, 3.8)


def test_oracle_anderson_beats_simple_mixing(orc):
    # the same lamellar start: Anderson reaches 1e-4 quickly, simple mixing does not
    p = P(orc, nx=16, ny=4, nz=4, lx=4.0, hAB=15.0, fA=0.5, ds0=0.02)
    x = np.arange(p.nx) * p.lx / p.nx
    base = 1.5 * np.cos(2 * np.pi * x / p.lx) * np.ones(p.shape)
    rng = np.random.default_rng(0)
    wa = base[None] + rng.normal(0, 0.01, (1,) + p.shape)
    wb = -base[None] + rng.normal(0, 0.01, (1,) + p.shape)
    ra = orc.converge_loop(wa, wb, p, 1e-4, 300, mixing="anderson", m=10, lam=0.5, start=0.1)
    rs = orc.converge_loop(wa, wb, p, 1e-4, 300, mixing="simple")
    assert ra[6][-1] < 1e-4
    assert ra[5] < rs[5] or rs[6][-1] > 1e-4
    # at the saddle point incompressibility holds and the residual vanishes
    _, _, emax, _, _, _ = orc.residual(ra[0], ra[1], ra[2], ra[3], p.hAB, p.wcmp)
    assert emax[0] < 1e-3


def test_analytic_stress_matches_finite_differences(orc):
    """The spectral stress formula (q, q+ contracted with d exp(-ds k^2)/dL)
    equals central differences of -ln Q with h = 1e-4 L, including the
    constant wave number of a length-1 axis."""
    rng = np.random.default_rng(1)
    for grid in ((12, 8, 6), (12, 8, 1)):
        p = orc.Params(nx=grid[0], ny=grid[1], nz=grid[2], lx=3.1, ly=2.7, lz=2.2, hAB=15.0,
                       fA=0.4, ds0=0.05, batch=2)
        wa = rng.normal(0, 1.5, (2,) + p.shape)
        wb = rng.normal(0, 1.5, (2,) + p.shape)
        a = orc.stress_spectral(wa, wb, p)
        b = orc.stress_fd(wa, wb, p)
        assert np.abs(a - b).max() < 1e-7 * np.abs(a).max()


def test_contour_weights(orc):
    """Trapezoid weights are the reference's (w_to_phi_go, cuda_aid.cu:87-107);
    the Simpson weights of a block of n >= 1 steps sum to n and integrate
    cubics exactly (the 1/3 rule and, for odd n, the 3/8 rule at the end)."""
    assert list(orc.contour_weights(0)) == [0.5] == list(orc.contour_weights(0, True))
    assert list(orc.contour_weights(4)) == [0.5, 1, 1, 1, 0.5]
    assert list(orc.contour_weights(1, True)) == [0.5, 0.5]
    for n in range(2, 40):
        w = orc.contour_weights(n, True)
        s = np.arange(n + 1.0)
        for k in range(4):
            assert abs((w * s ** k).sum() - n ** (k + 1) / (k + 1)) < 1e-12 * n ** (k + 1)
    rng = np.random.default_rng(0)
    q, qc = rng.random((2, 2, 8, 3, 4))
    np.testing.assert_allclose(orc.contour_sum(q, qc), orc.trapezoid_sum(q, qc), rtol=1e-15)


def test_remove_translation_removes_a_pure_shift():
    """An update that is a small rigid shift of the fields (plus nothing else)
    is removed to first order; an update orthogonal to the shifts is kept."""
    from oracle import scft_oracle as orc
    n = 16
    x = np.arange(n) * 2 * np.pi / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    wa = (np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X))[None]
    wb = -wa
    ta = orc.translation_generators(wa)
    tb = orc.translation_generators(wb)
    d = 1e-3
    a1, b1 = orc.remove_translation(wa, wb, wa - d * (ta[0] + 2 * ta[1]),
                                    wb - d * (tb[0] + 2 * tb[1]))
    assert np.abs(a1 - wa).max() < 1e-14 and np.abs(b1 - wb).max() < 1e-14
    # the uniform field is orthogonal to every central difference
    a2, b2 = orc.remove_translation(wa, wb, wa + 0.5, wb - 0.25)
    assert np.allclose(a2 - wa, 0.5, atol=1e-14) and np.allclose(b2 - wb, -0.25, atol=1e-14)
    # a length-1 axis has no generator
    assert orc.translation_generators(wa[:, :1])[2] is None
