"""Constrained field updates and the VTK export on the GPU, through the C ABI.

phi_w_constrained / phi_w_constrainedEx (cuda_aid.cu:418-490) are pointwise
FP64 updates: the kernels must match the oracle to rounding (1e-13 relative)
and the reference's own kernels (golden fixture, run on a GB300) to the same
bound.  The constrained SCF loop (mixing SCFT_MIX_CONSTRAINED[_EX]) is
checked against the oracle's loop to the FP64 path's 1e-11."""
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_constrained16x12x8.npz")


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_constrained_kernels_match_reference_and_oracle(pkg, orc):
    g = np.load(GOLD)
    nx, ny, nz = (int(v) for v in g["grid"])
    lx, ly, lz = (float(v) for v in g["box"])
    chiN, lam = float(g["chiN"]), float(g["lam"])
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=chiN, fA=0.5, ds0=0.05,
                     batch=2) as ctx:
        ctx.set_target(g["target"])
        for key, ex in (("con", False), ("conex", True)):
            ctx.set_w(g["wa_in"], g["wb_in"])
            ctx.set_field(pkg.FIELD_PHA, g["pha"])
            ctx.set_field(pkg.FIELD_PHB, g["phb"])
            ctx.phi_w_constrained(ex, lam)
            if ex:
                owa, owb = orc.phi_w_constrained_ex(g["wa_in"], g["wb_in"], g["pha"], g["phb"],
                                                    g["target"], chiN)
            else:
                owa, owb = orc.phi_w_constrained(g["wa_in"], g["wb_in"], g["pha"], g["phb"],
                                                 g["target"], chiN, lam)
            for dev, ref, o in ((ctx.wa, g[key + "_wa"], owa), (ctx.wb, g[key + "_wb"], owb)):
                assert rel(dev, ref) < 1e-13
                assert rel(dev, o) < 1e-13


@pytest.mark.parametrize("ex", [False, True])
def test_constrained_loop_matches_oracle(pkg, orc, ex):
    from scft_gb300 import fields
    nx, ny, nz, L = 16, 16, 8, (4.0, 4.0, 2.0)
    wa, wb = fields.lamellar(nx, ny, nz, *L, 20.0, seed=5, batch=2)
    rng = np.random.default_rng(9)
    x = (np.arange(nx) + 0.5) / nx
    target = np.broadcast_to(0.5 + 0.4 * np.cos(2 * np.pi * x), (2, nz, ny, nx)).copy()
    target += rng.normal(0, 0.01, target.shape)
    lam = 0.0 if ex else 1.5
    mixing = pkg.MIX_CONSTRAINED_EX if ex else pkg.MIX_CONSTRAINED
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=L[0], ly=L[1], lz=L[2], hAB=20.0, fA=0.5,
                     ds0=0.02, batch=2, mixing=mixing, constraint_lambda=lam) as ctx:
        ctx.set_w(wa, wb)
        ctx.set_target(target)
        ctx.iterate(4)
        dev_wa, dev_wb, dev_pha = ctx.wa, ctx.wb, ctx.pha
        mx, _ = ctx.residual()
    p = orc.Params(nx=nx, ny=ny, nz=nz, lx=L[0], ly=L[1], lz=L[2], hAB=20.0, fA=0.5, ds0=0.02,
                   batch=2)
    for _ in range(4):
        wa = orc.average_value(wa)
        wb = orc.average_value(wb)
        c = orc.get_conc(wa, wb, p)
        if ex:
            wa, wb = orc.phi_w_constrained_ex(c.wa, wb, c.pha, c.phb, target, p.hAB)
        else:
            wa, wb = orc.phi_w_constrained(c.wa, wb, c.pha, c.phb, target, p.hAB, lam)
    assert rel(dev_wa, wa) < 1e-11
    assert rel(dev_wb, wb) < 1e-11
    assert rel(dev_pha, c.pha) < 1e-11
    assert np.all(np.isfinite(mx)) and np.all(mx > 0)


def test_constrained_needs_target(pkg):
    with pkg.Context(nx=8, ny=8, nz=8) as ctx:
        with pytest.raises(pkg.ScftError):
            ctx.phi_w_constrained(False, 1.0)
    with pkg.Context(nx=8, ny=8, nz=8, mixing=pkg.MIX_CONSTRAINED) as ctx:
        with pytest.raises(pkg.ScftError):
            ctx.iterate(1)


def test_write_vtk_equals_pha_file_route(pkg, orc, tmp_path, monkeypatch):
    from scft_gb300 import fields
    monkeypatch.chdir(tmp_path)
    nx, ny, nz = 24, 16, 8
    wa, wb = fields.gyroid(nx, ny, nz, 3.8, 3.8, 3.8, 18.0, seed=3, batch=2)
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=3.8, ly=3.8, lz=3.8, hAB=18.0, fA=0.36,
                     ds0=0.02, batch=2) as ctx:
        ctx.set_w(wa, wb)
        ctx.iterate(3)
        ctx.write_vtk("direct.vtk", 1, "pha_2.dat")
        ctx.write_pha_dat("pha_2.dat", 1)
    pkg.convert_pha_to_vtk("pha_2.dat", "converted.vtk")
    direct = open("direct.vtk", "rb").read()
    assert direct == open("converted.vtk", "rb").read()
    assert direct.decode() == orc.convert_pha_to_vtk("pha_2.dat")
    assert hashlib.sha256(direct).hexdigest()
