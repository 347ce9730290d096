"""Pin the CPU oracle to the reference: golden vectors produced by the
reference's own kernels + cuFFT on a GB300 (tests/golden/make_ref_golden.py)
must be reproduced by the oracle on the CPU."""
import glob
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# SCF cases (getConc + loop); the quirk, constrained-update and VTK fixtures
# have their own tests
CASES = sorted(p for p in glob.glob(os.path.join(GOLD, "ref_*.npz"))
               if "loop_fe" in np.load(p).files)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def params(orc, d):
    nx, ny, nz = (int(v) for v in d["grid"])
    lx, ly, lz = (float(v) for v in d["box"])
    return orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=float(d["chiN"]),
                      fA=float(d["fA"]), ds0=float(d["ds0"]), batch=int(d["batch"]))


def test_fixtures_present():
    assert len(CASES) >= 5, "reference golden vectors missing: run tests/golden/make_ref_golden.py"


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c) for c in CASES])
def test_oracle_get_conc_matches_reference(orc, path):
    d = np.load(path)
    p = params(orc, d)
    c = orc.get_conc(d["wa_in"], d["wb_in"], p)
    assert rel(c.wa, d["conc_wa"]) < 1e-13
    assert rel(c.pha, d["conc_pha"]) < 1e-11
    assert rel(c.phb, d["conc_phb"]) < 1e-11
    assert np.abs(c.Q / d["conc_Q"] - 1).max() < 1e-11
    assert rel(c.qa[:, p.NsA], d["qa_end"]) < 1e-11
    assert rel(c.qcb[:, 0], d["qcb_0"]) < 1e-11
    assert rel(c.qb[:, p.dNsB], d["qb_end"]) < 1e-11
    assert rel(c.qca[:, 0], d["qca_0"]) < 1e-11
    assert rel(c.qca[:, p.NsA // 2], d["qca_mid"]) < 1e-11


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c) for c in CASES])
def test_oracle_free_loop_matches_reference(orc, path):
    d = np.load(path)
    p = params(orc, d)
    res = orc.free_loop(d["wa_in"], d["wb_in"], p, int(d["iters"]))
    assert rel(res.wa, d["loop_wa"]) < 1e-10
    assert rel(res.wb, d["loop_wb"]) < 1e-10
    assert rel(res.pha, d["loop_pha"]) < 1e-10
    assert np.abs(res.Q / d["loop_Q"] - 1).max() < 1e-10
    fe = np.stack(orc.free_energy(res.wa, res.wb, res.pha, res.phb, res.Q, p.hAB), axis=1)
    np.testing.assert_allclose(fe, d["loop_fe"], rtol=1e-10, atol=1e-12)


def test_reduce3_quirk_matches_reference(orc):
    path = os.path.join(GOLD, "ref_quirk12.npz")
    d = np.load(path)
    w = d["w_in"]
    M = w.size
    T = orc.factor_decompose_1024(M)
    assert T == 864
    mean_quirk = orc.reduce3_quirk_sum(w.ravel(), T) / M
    np.testing.assert_allclose(d["w_avg"], w - mean_quirk, rtol=0, atol=1e-13)
    # ... and it is not the true mean subtraction
    assert np.abs(d["w_avg"] - orc.average_value(w)).max() > 1e-6


def test_constrained_updates_match_reference(orc):
    """phi_w_constrained (lambda 0.7) and phi_w_constrainedEx run by the
    reference's own kernels (cuda_aid.cu:418-490) on seeded fields."""
    d = np.load(os.path.join(GOLD, "ref_constrained16x12x8.npz"))
    chiN, lam = float(d["chiN"]), float(d["lam"])
    args = (d["wa_in"], d["wb_in"], d["pha"], d["phb"], d["target"], chiN)
    wa, wb = orc.phi_w_constrained(*args, lam)
    assert rel(wa, d["con_wa"]) < 1e-14 and rel(wb, d["con_wb"]) < 1e-14
    wa, wb = orc.phi_w_constrained_ex(*args)
    assert rel(wa, d["conex_wa"]) < 1e-14 and rel(wb, d["conex_wb"]) < 1e-14
    # the penalty term is really exercised
    wa0, _ = orc.phi_w_constrained(*args, 0.0)
    assert rel(wa0, d["con_wa"]) > 1e-3
