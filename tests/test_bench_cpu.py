"""The benchmark's own measurement helpers (no GPU): the rigid-shift
alignment used to compare converged structures, and the agreement summary
of two converged runs."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test",
                                                  os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def field(shape, shift=(0.0, 0.0, 0.0)):
    """A smooth periodic structure sampled at r - shift (shift in voxels)."""
    axes = [2 * np.pi * (np.arange(n) - s) / n for n, s in zip(shape, shift)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    return 0.4 + 0.2 * (np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X))


def test_alignment_recovers_a_subvoxel_shift():
    b = load_bench()
    shape = (24, 20, 16)
    a = field(shape)
    shifted = field(shape, (0.013, -0.021, 0.007))
    raw = np.abs(a - shifted).max() / np.abs(a).max()
    al, d = b.translation_aligned_diff(a, shifted)
    assert raw > 1e-3
    assert al < 1e-9
    # b(r - d) = a(r): the fitted shift undoes the applied one
    np.testing.assert_allclose(d, [-0.013, 0.021, -0.007], atol=1e-9)


def test_alignment_keeps_a_real_difference():
    b = load_bench()
    shape = (16, 16, 16)
    a = field(shape)
    other = a + 1e-4 * np.cos(2 * np.pi * 2 * np.arange(16) / 16)[:, None, None]
    al, _ = b.translation_aligned_diff(a, other)
    assert al > 1e-5          # a change of shape is not a translation


def test_compare_to_fp64_summary():
    b = load_bench()
    shape = (16, 16, 16)
    pa = field(shape)[None]
    pb = 1.0 - pa
    ref = (pa, pb, np.array([2.0]), 3.5)
    run = (field(shape, (0.01, 0.0, 0.0))[None], 1.0 - field(shape, (0.01, 0.0, 0.0))[None],
           np.array([2.0 + 2e-9]), 3.5 + 1e-9)
    out = b.compare_to_fp64(ref, run)
    assert abs(out["F_abs_diff"] - 1e-9) < 1e-15
    assert abs(out["Q_rel_diff"] - 1e-9) < 1e-15
    assert out["phiA_rel_diff"] > 1e-4
    assert out["phiA_rel_diff_shift_aligned"] < 1e-9
    assert out["phiB_rel_diff_shift_aligned"] < 1e-9
    assert out["phiA_spectrum_rel_diff"] < 1e-12
