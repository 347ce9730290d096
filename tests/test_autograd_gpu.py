"""Gradient-check harness: the torch.autograd.Function over getConc and its
CUDA adjoint (FP64 context) against finite differences.

- torch.autograd.gradcheck (random-projection mode) of (wA, wB, box) ->
  (phiA, phiB, Q), FD of the CUDA forward itself;
- dF/dL of the free energy against central differences of the oracle's F with
  h = 1e-4 L, and dF/dw along random directions (2e-6 relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def setup(pkg, orc, grid=(10, 8, 6), box=(3.1, 2.7, 2.2), fA=0.4, ds0=0.05, batch=1):
    nx, ny, nz = grid
    ctx = pkg.Context(nx=nx, ny=ny, nz=nz, lx=box[0], ly=box[1], lz=box[2], hAB=15.0, fA=fA,
                      ds0=ds0, batch=batch)
    p = orc.Params(nx=nx, ny=ny, nz=nz, lx=box[0], ly=box[1], lz=box[2], hAB=15.0, fA=fA,
                   ds0=ds0, batch=batch)
    rng = np.random.default_rng(5)
    wa = rng.normal(0, 1.5, (batch,) + p.shape)
    wb = rng.normal(0, 1.5, (batch,) + p.shape)
    return ctx, p, wa, wb


def test_gradcheck_get_conc(pkg, orc):
    from scft_gb300.autograd import GetConc
    ctx, p, wa, wb = setup(pkg, orc, grid=(8, 6, 4), ds0=0.1)
    with ctx:
        ta = torch.tensor(wa, requires_grad=True)
        tb = torch.tensor(wb, requires_grad=True)
        box = torch.tensor([p.lx, p.ly, p.lz], dtype=torch.float64, requires_grad=True)
        f = lambda a, b, L: GetConc.apply(a, b, L, ctx, 2)
        assert torch.autograd.gradcheck(f, (ta, tb, box), eps=1e-6, atol=1e-6, rtol=1e-5,
                                        fast_mode=True)


def test_free_energy_gradients_match_oracle_fd(pkg, orc):
    from scft_gb300.autograd import free_energy
    ctx, p, wa, wb = setup(pkg, orc, batch=2)
    with ctx:
        ta = torch.tensor(wa, requires_grad=True)
        tb = torch.tensor(wb, requires_grad=True)
        box = torch.tensor([p.lx, p.ly, p.lz], dtype=torch.float64, requires_grad=True)
        F = free_energy(ta, tb, box, ctx, p.hAB)
        F_dev = F.detach().numpy().copy()
        F.sum().backward()
    # the forward is the oracle's F
    assert np.abs(F_dev - orc.free_energy_of(wa, wb, p)).max() < 1e-11
    Fsum = lambda a, b, pp: float(orc.free_energy_of(a, b, pp).sum())
    lens = (p.lx, p.ly, p.lz)
    for a in range(3):
        h = 1e-4 * lens[a]
        Lp, Lm = list(lens), list(lens)
        Lp[a] += h
        Lm[a] -= h
        fd = (Fsum(wa, wb, orc.with_box(p, *Lp)) - Fsum(wa, wb, orc.with_box(p, *Lm))) / (2 * h)
        ad = float(box.grad[a])
        assert abs(ad - fd) < 2e-6 * max(abs(fd), 1e-3), (a, ad, fd)
    rng = np.random.default_rng(8)
    for _ in range(2):
        dA, dB = rng.normal(0, 1, wa.shape), rng.normal(0, 1, wa.shape)
        h = 1e-5
        fd = (Fsum(wa + h * dA, wb + h * dB, p) - Fsum(wa - h * dA, wb - h * dB, p)) / (2 * h)
        ad = float((ta.grad.numpy() * dA).sum() + (tb.grad.numpy() * dB).sum())
        assert abs(ad - fd) < 2e-6 * max(abs(fd), 1e-3), (ad, fd)
