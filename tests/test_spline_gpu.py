"""Batched spline evaluation on the GPU equals the host evaluation (and so
the reference's seval/deriv/sinteg) bit for bit: explicitly rounded device
arithmetic, the same segment search."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n,e1,e2", [(2, 0, 0), (3, 0, 0), (50, 0, 0), (50, 1, 1)])
def test_device_eval_equals_host(pkg, n, e1, e2):
    rng = np.random.default_rng(n)
    x = np.cumsum(rng.uniform(0.1, 1.0, n))
    y = np.cos(x)
    sp = pkg.Spline(x, y, e1, e2, 0.3, -0.2)
    u = np.concatenate([rng.uniform(x[0] - 1, x[-1] + 1, 20000), x])
    ut = torch.tensor(u, device="cuda:0")
    for mode, f in ((0, sp), (1, sp.deriv), (2, sp.integral)):
        dev = sp.eval_device(ut, mode).cpu().numpy()
        host = np.empty_like(u)
        for k, uk in enumerate(u):
            sp.last.value = 0          # the device starts every search from segment 0
            host[k] = f(uk)
        assert np.array_equal(dev, host), mode
