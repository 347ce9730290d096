"""Binary checkpoint (exact resume) and JSON-lines progress metrics.

A run saved after k iterations and resumed in a fresh context must repeat
the uninterrupted run bit for bit, with simple mixing and with Anderson
mixing (whose history ring, Gram matrix and iteration count are part of the
state)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# Nx = 64 so that the double-float path (register kernels on every axis) runs too
G = dict(nx=64, ny=32, nz=32, lx=7.6, ly=3.8, lz=3.8, hAB=18.0, fA=0.36, ds0=0.01)


def start_fields(batch=2):
    from scft_gb300 import fields as fl
    return fl.gyroid(G["nx"], G["ny"], G["nz"], G["lx"], G["ly"], G["lz"], G["hAB"], seed=3,
                     batch=batch)


def ctx_kw(pkg, prec, mixing, **extra):
    kw = dict(G, batch=2, precision={"fp32": pkg.PREC_FP32, "df": pkg.PREC_DF}.get(
        prec, pkg.PREC_FP64))
    if mixing == "anderson":
        kw.update(mixing=pkg.MIX_ANDERSON, anderson_history=5, anderson_start=1e9)
    kw.update(extra)
    return kw


@pytest.mark.parametrize("mixing", ["simple", "anderson"])
@pytest.mark.parametrize("prec", ["fp64", "fp32", "df"])
def test_resume_repeats_the_run_bit_for_bit(pkg, tmp_path, prec, mixing):
    wa, wb = start_fields()
    path = tmp_path / "run.ckpt"
    kw = ctx_kw(pkg, prec, mixing)
    with pkg.Context(**kw) as a:
        a.set_w(wa, wb)
        a.iterate(12)                 # Anderson: the 6-slot ring has wrapped
        a.save_checkpoint(path)
        a.iterate(9)
        ref = [a.wa, a.wb, a.pha, a.phb, a.residual()[0], a.free_energy()]
    with pkg.Context(**kw) as b:
        b.load_checkpoint(path)
        b.iterate(9)
        got = [b.wa, b.wb, b.pha, b.phb, b.residual()[0], b.free_energy()]
    for r, g in zip(ref, got):
        assert np.array_equal(r, g)


def test_history_restarts_when_the_operator_differs(pkg, tmp_path):
    wa, wb = start_fields()
    path = tmp_path / "run.ckpt"
    with pkg.Context(**ctx_kw(pkg, "fp64", "anderson")) as a:
        a.set_w(wa, wb)
        a.iterate(8)
        a.save_checkpoint(path)
        w_saved = (a.wa, a.wb, a.pha)
    # another chi N: the fields load, the history (of the other operator) does not
    with pkg.Context(**ctx_kw(pkg, "fp64", "anderson", hAB=17.5)) as b:
        b.load_checkpoint(path)
        assert np.array_equal(b.wa, w_saved[0]) and np.array_equal(b.pha, w_saved[2])
        b.iterate(3)
        assert np.isfinite(b.residual()[0]).all()
    # fields only (no history in the file) into a simple-mixing context
    with pkg.Context(**ctx_kw(pkg, "fp64", "anderson")) as a:
        a.set_w(wa, wb)
        a.iterate(2)
        a.save_checkpoint(path, with_history=False)
        w2 = a.wb
    with pkg.Context(**ctx_kw(pkg, "fp32", "simple")) as c:
        c.load_checkpoint(path)
        assert np.array_equal(c.wb, w2)


def test_history_restarts_when_lambda_differs(pkg, tmp_path):
    """The ring holds u = w + lambda d, so a history saved with another lambda
    is not reused: the resumed run equals one loaded without any history."""
    wa, wb = start_fields()
    with_h, without_h = tmp_path / "h.ckpt", tmp_path / "n.ckpt"
    with pkg.Context(**ctx_kw(pkg, "fp64", "anderson")) as a:
        a.set_w(wa, wb)
        a.iterate(8)
        a.save_checkpoint(with_h)
        a.save_checkpoint(without_h, with_history=False)
    runs = []
    for path in (with_h, without_h):
        with pkg.Context(**ctx_kw(pkg, "fp64", "anderson", anderson_lambda=0.4)) as b:
            b.load_checkpoint(path)
            b.iterate(5)
            runs.append((b.wa, b.wb))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_checkpoint_errors(pkg, tmp_path):
    wa, wb = start_fields()
    path = tmp_path / "run.ckpt"
    with pkg.Context(**ctx_kw(pkg, "fp64", "simple")) as a:
        a.set_w(wa, wb)
        a.save_checkpoint(path)
    with pkg.Context(**dict(ctx_kw(pkg, "fp64", "simple"), nz=16, lz=1.9)) as b:
        with pytest.raises(pkg.ScftError) as e:
            b.load_checkpoint(path)
        assert e.value.status == pkg.ERR_INVALID_ARG
        bad = tmp_path / "bad.ckpt"
        bad.write_bytes(b"not a checkpoint at all")
        with pytest.raises(pkg.ScftError) as e:
            b.load_checkpoint(bad)
        assert e.value.status == pkg.ERR_IO
        with pytest.raises(pkg.ScftError) as e:
            b.load_checkpoint(tmp_path / "missing.ckpt")
        assert e.value.status == pkg.ERR_IO
    # a truncated file (the fields are short) or one with trailing bytes: an
    # error, and the context's fields are unchanged (the file is checked
    # whole before anything reaches the device)
    data = path.read_bytes()
    short = tmp_path / "short.ckpt"
    long_ = tmp_path / "long.ckpt"
    short.write_bytes(data[: len(data) // 2])
    long_.write_bytes(data + b"\0" * 8)
    with pkg.Context(**ctx_kw(pkg, "fp64", "simple")) as c:
        w0 = [x + 0.25 for x in start_fields()]
        c.set_w(*w0)
        for f in (short, long_):
            with pytest.raises(pkg.ScftError) as e:
                c.load_checkpoint(f)
            assert e.value.status == pkg.ERR_IO
            assert np.array_equal(c.wa, w0[0]) and np.array_equal(c.wb, w0[1])


def test_truncated_history_leaves_the_context_unchanged(pkg, tmp_path):
    """A checkpoint cut inside its Anderson history: the load fails before
    any field or history slot is touched, and the run continues exactly as
    it would have without the attempt."""
    wa, wb = start_fields()
    path = tmp_path / "run.ckpt"
    kw = ctx_kw(pkg, "fp64", "anderson")
    with pkg.Context(**kw) as a:
        a.set_w(wa, wb)
        a.iterate(7)
        a.save_checkpoint(path)
    data = path.read_bytes()
    cut = tmp_path / "cut.ckpt"
    cut.write_bytes(data[: len(data) - 1000])
    with pkg.Context(**kw) as b, pkg.Context(**kw) as ref:
        for c in (b, ref):
            c.set_w(wa + 0.1, wb - 0.1)
            c.iterate(4)
        with pytest.raises(pkg.ScftError) as e:
            b.load_checkpoint(cut)
        assert e.value.status == pkg.ERR_IO
        b.iterate(3)
        ref.iterate(3)
        assert np.array_equal(b.wa, ref.wa) and np.array_equal(b.wb, ref.wb)


def test_free_writes_json_lines(pkg, tmp_path, capfd):
    wa, wb = start_fields()
    path = tmp_path / "metrics.jsonl"
    with pkg.Context(**ctx_kw(pkg, "fp64", "simple")) as ctx:
        ctx.set_w(wa, wb)
        ctx.set_metrics_file(str(path))
        ctx.free(20, 10)
        fe = ctx.free_energy()
        mx, rms = ctx.residual()
        ctx.set_metrics_file(None)
        ctx.free(10, 10)              # off again: nothing appended
    rows = [json.loads(line) for line in path.read_text().splitlines()]
    assert [(r["iteration"], r["instance"]) for r in rows] == [(10, 0), (10, 1), (20, 0), (20, 1)]
    keys = {"F", "F_AB", "F_W", "F_S", "inCompMax", "residual_max", "residual_rms", "elapsed_s"}
    assert all(keys <= set(r) for r in rows)
    for i in range(2):
        last = rows[2 + i]
        np.testing.assert_allclose([last["F"], last["F_AB"], last["F_W"], last["F_S"],
                                    last["inCompMax"]], fe[i], rtol=1e-14, atol=1e-15)
        assert last["residual_max"] == mx[i] and last["residual_rms"] == rms[i]
    assert rows[2]["elapsed_s"] >= rows[0]["elapsed_s"] >= 0
    out = capfd.readouterr().out     # the reference's progress lines are unchanged
    assert out.count("GPU 0 batch 0:") == 3
