"""Failure detection without a GPU fault (host-side injection and a bounded
device wait): every failure is a status code, and the device stays usable."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def usable(pkg):
    with pkg.Context(nx=16, ny=16, nz=16) as ctx:
        z = np.zeros(ctx.shape)
        ctx.set_w(z, z)
        ctx.get_conc()
        return abs(ctx.Q()[0] - 1.0) < 1e-12


def test_bounded_wait_times_out_and_reports(pkg):
    lib = pkg.load_library()
    t = C.c_int(-1)
    assert lib.scft_selftest_bounded_wait(0, 0.05, C.byref(t)) == pkg.OK
    assert t.value == 1
    assert usable(pkg)


def test_allocation_failure_is_reported(pkg):
    # 4096^3 points: the first field alone is 550 GB
    with pytest.raises(pkg.ScftError) as e:
        pkg.Context(nx=4096, ny=4096, nz=4096)
    assert e.value.status == pkg.ERR_NO_MEMORY
    assert usable(pkg)


def test_diverging_iteration_is_reported(pkg):
    """A mixing step far too large makes the fields blow up: converge stops
    with SCFT_ERR_NOT_FINITE instead of running on NaNs."""
    from scft_gb300 import fields
    wa, wb = fields.lamellar(16, 16, 16, 4.0, 4.0, 4.0, 20.0, seed=1)
    with pkg.Context(nx=16, ny=16, nz=16, wopt=50.0) as ctx:
        ctx.set_w(wa, wb)
        with pytest.raises(pkg.ScftError) as e:
            ctx.converge(1e-8, 2000)
        assert e.value.status == pkg.ERR_NOT_FINITE
    assert usable(pkg)


@pytest.mark.parametrize("mixing", ["simple", "anderson"])
def test_nan_field_is_reported_not_converged(pkg, mixing):
    """One NaN point spreads through the propagators to every point; the
    residual max-norm must come out NaN (a plain fmax reduction drops NaNs
    and would report 0, i.e. converged), so converge stops at the first
    check with SCFT_ERR_NOT_FINITE."""
    from scft_gb300 import fields
    wa, wb = fields.lamellar(16, 16, 16, 4.0, 4.0, 4.0, 20.0, seed=2)
    wa.reshape(-1)[123] = np.nan
    kw = {"mixing": pkg.MIX_ANDERSON, "anderson_history": 5} if mixing == "anderson" else {}
    with pkg.Context(nx=16, ny=16, nz=16, **kw) as ctx:
        ctx.set_w(wa, wb)
        with pytest.raises(pkg.ScftError) as e:
            ctx.converge(1e-6, 5)
        assert e.value.status == pkg.ERR_NOT_FINITE
        mx, rms = ctx.residual()
        assert np.isnan(mx[0]) and np.isnan(rms[0])
    assert usable(pkg)
