"""Heterogeneous batched sweeps: a group of contexts with different grids and
parameters advanced by one CUDA-graph launch per iteration gives exactly the
fields each context reaches on its own (the kernels and reduction orders are
the same; only their concurrency changes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MEMBERS = [
    dict(nx=32, ny=32, nz=32, lx=4.0, ly=4.0, lz=4.0, hAB=20.0, fA=0.5, ds0=0.01),
    dict(nx=48, ny=48, nz=48, lx=3.8, ly=3.8, lz=3.8, hAB=18.0, fA=0.36, ds0=0.005),
    dict(nx=64, ny=64, nz=64, lx=4.5, ly=4.5, lz=4.5, hAB=25.0, fA=0.3, ds0=0.0075),
    dict(nx=64, ny=32, nz=16, lx=4.2, ly=3.0, lz=2.0, hAB=15.0, fA=0.45, ds0=0.02, batch=2),
]


def start_fields(kw, seed):
    from scft_gb300 import fields
    return fields.gyroid(kw["nx"], kw["ny"], kw["nz"], kw["lx"], kw["ly"], kw["lz"], kw["hAB"],
                         seed=seed, batch=kw.get("batch", 1))


@pytest.mark.parametrize("mixing", [0, 1])
def test_group_equals_individual(pkg, mixing):
    extra = dict(precision=pkg.PREC_FP32, mixing=mixing, anderson_history=8)
    solo = []
    for i, kw in enumerate(MEMBERS):
        with pkg.Context(**kw, **extra) as ctx:
            ctx.set_w(*start_fields(kw, i))
            ctx.iterate(6)
            solo.append((ctx.wa, ctx.pha))
    ctxs = [pkg.Context(**kw, **extra) for kw in MEMBERS]
    for i, (ctx, kw) in enumerate(zip(ctxs, MEMBERS)):
        ctx.set_w(*start_fields(kw, i))
    with pkg.Group(ctxs) as g:
        g.iterate(6)
        assert g.launch_count() > 0
    for ctx, (wa, pha) in zip(ctxs, solo):
        assert np.array_equal(ctx.wa, wa)
        assert np.array_equal(ctx.pha, pha)
    for ctx in ctxs:
        ctx.close()


def test_group_mixes_precisions_and_rules(pkg):
    """Members may differ in propagation precision (FP32, FP64, double-float)
    and contour rule; each still reaches exactly its own solo result."""
    members = [
        dict(MEMBERS[0], precision=pkg.PREC_FP64),
        dict(MEMBERS[2], precision=pkg.PREC_DF, flags=pkg.FLAG_SIMPSON),
        dict(MEMBERS[3], precision=pkg.PREC_FP32, mixing=1, anderson_history=4),
        dict(MEMBERS[3], nz=32, lz=4.0, precision=pkg.PREC_DF),
    ]
    solo = []
    for i, kw in enumerate(members):
        with pkg.Context(**kw) as ctx:
            ctx.set_w(*start_fields(kw, i))
            ctx.iterate(4)
            solo.append((ctx.wb, ctx.phb))
    ctxs = [pkg.Context(**kw) for kw in members]
    for i, (ctx, kw) in enumerate(zip(ctxs, members)):
        ctx.set_w(*start_fields(kw, i))
    with pkg.Group(ctxs) as g:
        g.iterate(4)
    for ctx, (wb, phb) in zip(ctxs, solo):
        assert np.array_equal(ctx.wb, wb)
        assert np.array_equal(ctx.phb, phb)
    for ctx in ctxs:
        ctx.close()


@pytest.mark.parametrize("grid", [(64, 64, 64), (128, 64, 32)])
def test_autotuned_schedule_gives_same_results(pkg, grid):
    from scft_gb300 import fields
    nx, ny, nz = grid
    kw = dict(nx=nx, ny=ny, nz=nz, lx=4.0, ly=4.0, lz=4.0, hAB=18.0, fA=0.36, ds0=0.01,
              precision=pkg.PREC_FP32)
    wa, wb = fields.gyroid(nx, ny, nz, 4.0, 4.0, 4.0, 18.0, seed=2)
    out = []
    for flags in (0, pkg.FLAG_AUTOTUNE):
        with pkg.Context(flags=flags, **kw) as ctx:
            sched, ms = ctx.schedule()
            assert bool(sched & pkg.FLAG_TWO_STREAMS) != bool(sched & pkg.FLAG_LOCKSTEP)
            if flags:
                assert ms > 0
            ctx.set_w(wa, wb)
            ctx.iterate(2)
            out.append(ctx.pha)
    # schedules only reorder independent work: identical kernels per pass type,
    # so the results agree to FP32 round-off of the differing pass kernels
    assert np.abs(out[0] - out[1]).max() < 2e-5 * np.abs(out[0]).max()


def test_group_rejects_duplicates(pkg):
    kw = MEMBERS[0]
    with pkg.Context(**kw) as ctx:
        with pytest.raises(pkg.ScftError):
            pkg.Group([ctx, ctx])
