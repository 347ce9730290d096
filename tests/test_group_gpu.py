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


# same-grid FP32 members below 2^16 points or without fused step pairs form
# buckets whose marches run as one lockstep batched march (here 32^3 on the
# register kernels and 40^3 on the generic Stockham kernel); the rest keep
# their own schedules
BUCKETED = [
    dict(nx=64, ny=64, nz=64, lx=4.5, ly=4.5, lz=4.5, hAB=25.0, fA=0.3, ds0=0.0075),
    dict(nx=64, ny=64, nz=64, lx=3.8, ly=3.8, lz=3.8, hAB=18.0, fA=0.36, ds0=0.01),
    dict(nx=40, ny=40, nz=40, lx=3.8, ly=3.8, lz=3.8, hAB=18.0, fA=0.36, ds0=0.005),
    dict(nx=40, ny=40, nz=40, lx=4.4, ly=4.4, lz=4.4, hAB=22.0, fA=0.27, ds0=1 / 150),
    dict(nx=40, ny=40, nz=40, lx=3.2, ly=3.2, lz=3.2, hAB=14.0, fA=0.45, ds0=1 / 130),
    dict(nx=32, ny=32, nz=32, lx=4.0, ly=4.0, lz=4.0, hAB=20.0, fA=0.5, ds0=0.01),
    dict(nx=32, ny=32, nz=32, lx=3.1, ly=3.1, lz=3.1, hAB=29.0, fA=0.25, ds0=1 / 110),
    dict(nx=32, ny=32, nz=32, lx=4.0, ly=4.0, lz=4.0, hAB=20.0, fA=0.5, ds0=0.01,
         precision=0),                         # FP64: not bucketed
    dict(nx=64, ny=32, nz=16, lx=4.2, ly=3.0, lz=2.0, hAB=15.0, fA=0.45, ds0=0.02),  # alone
]


@pytest.mark.parametrize("mixing", [0, 1])
def test_batched_march_members_match_oracle_and_solo(pkg, orc, mixing):
    """Every member of a group with batched buckets: its getConc of the first
    iteration against the oracle (FP32 tolerance), and its fields after six
    iterations against the same context run alone (the lockstep unfused
    schedule against the solo fused one: FP32 round-off only)."""
    members = [dict(dict(precision=1), **kw) for kw in BUCKETED]
    extra = dict(mixing=mixing, anderson_history=8)
    solo, solo_launches = [], 0
    for i, kw in enumerate(members):
        with pkg.Context(**kw, **extra) as ctx:
            ctx.set_w(*start_fields(kw, 10 + i))
            ctx.iterate(6)
            solo.append((ctx.wa, ctx.pha))
            solo_launches += ctx.launch_count()
    ctxs = [pkg.Context(**kw, **extra) for kw in members]
    for i, (ctx, kw) in enumerate(zip(ctxs, members)):
        ctx.set_w(*start_fields(kw, 10 + i))
    with pkg.Group(ctxs) as g:
        g.iterate(1)
        for i, (ctx, kw) in enumerate(zip(ctxs, members)):
            wa0, wb0 = start_fields(kw, 10 + i)
            p = orc.Params(**{k: v for k, v in kw.items() if k != "precision"})
            ref = orc.get_conc(orc.average_value(wa0), orc.average_value(wb0), p)
            # FP32: these members march up to 2 x 260 split steps (ds down to
            # 1/130); round-off grows with the step count, so the bound is twice
            # that of the 50-100-step parity tests
            tol = 1e-11 if kw["precision"] == 0 else 4e-5
            assert np.abs(ctx.pha - ref.pha).max() / np.abs(ref.pha).max() < tol, i
            assert np.abs(ctx.Q() / ref.Q - 1).max() < tol, i
        g.iterate(5)
        group_launches = g.launch_count() + sum(c.launch_count() for c in ctxs)
    for i, (ctx, (wa, pha)) in enumerate(zip(ctxs, solo)):
        assert np.abs(ctx.wa - wa).max() / np.abs(wa).max() < 2e-5, i
        assert np.abs(ctx.pha - pha).max() / np.abs(pha).max() < 2e-5, i
    # the batched buckets launch fewer kernels than the members alone (two or
    # three members per bucket here; the 64-member sweep of bench.py has ~21)
    assert group_launches < solo_launches
    for ctx in ctxs:
        ctx.close()
