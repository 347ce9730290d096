"""The drop-in driver of the struct API run as the reference binary is run:
a directory with ab.txt and phi_<i>.dat (init.cpp:81-94,
init_cuda.cu:435-456), flags -step=N; it prints the progress lines of Free
(cuda_scft.cu:221) and time=, and writes pha_<i>.dat (cuda_scft.cu:233-243)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "scft_ver1.01_gb300", "scft_gb300_driver")


def write_case(orc, d, p, wa, wb):
    with open(os.path.join(d, "ab.txt"), "w") as f:
        f.write("intag=1024\nxN=%g\nfa=%.3f\nlx=%.15g, ly=%.15g, lz=%.15g\n"
                "Nx=%d, Ny=%d, Nz=%d\nds0=%g\nbatch=%d\n"
                % (p.hAB, p.fA, p.lx, p.ly, p.lz, p.nx, p.ny, p.nz, p.ds0, p.batch))
    for i in range(p.batch):
        z = np.zeros(p.M)
        orc.write_pha_dat(os.path.join(d, "phi_%d.dat" % (i + 1)), p, z, z, wa[i].ravel(),
                          wb[i].ravel())


@pytest.mark.parametrize("prec,rtol", [("fp64", 1e-7), ("fp32", 2e-5)])
def test_driver_matches_oracle(pkg, orc, tmp_path, prec, rtol):
    assert os.path.exists(DRIVER), "driver not built"
    from scft_gb300 import fields
    p = orc.Params(nx=16, ny=16, nz=8, lx=4.0, ly=4.0, lz=2.0, hAB=20.0, fA=0.5, ds0=0.01,
                   batch=2)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=4, batch=2)
    d = str(tmp_path)
    write_case(orc, d, p, wa, wb)
    r = subprocess.run([DRIVER, "-step=100", "-precision=" + prec], cwd=d, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("GPU ")]
    assert len(lines) == 20                      # every 10 iterations x 2 instances
    assert any(l.startswith("time=") for l in r.stdout.splitlines())
    # the oracle starts from the same %g-rounded fields the driver read
    wa0 = np.stack([orc.read_phi_dat(os.path.join(d, "phi_%d.dat" % (i + 1)), p.M)[2]
                    for i in range(2)]).reshape((2,) + p.shape)
    wb0 = np.stack([orc.read_phi_dat(os.path.join(d, "phi_%d.dat" % (i + 1)), p.M)[3]
                    for i in range(2)]).reshape((2,) + p.shape)
    ref = orc.free_loop(wa0, wb0, p, 100)
    for l, row in zip(lines, ref.log):
        it, b, F, fab, fw, fs, inc = row
        assert l.startswith("GPU 0 batch %d: %5d :" % (b, it))
        vals = [float(v) for v in l.split(":")[2].split(",")]
        np.testing.assert_allclose(vals[:4], [F, fab, fw, fs], rtol=rtol, atol=1e-9)
    for i in range(2):
        path = os.path.join(d, "pha_%d.dat" % (i + 1))
        assert os.path.exists(path)
        head = open(path).read().splitlines()[:2]
        assert head[0] == "Nx=16, Ny=16, Nz=8"
        pa, pb, a, b = orc.read_phi_dat(path, p.M)
        np.testing.assert_allclose(pa, ref.pha[i].ravel(), rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(a, ref.wa[i].ravel(), rtol=1e-4, atol=1e-5)


def test_driver_optional_keys_and_metrics(pkg, orc, tmp_path):
    """ab.txt's optional lines switch the driver to Anderson mixing in FP32
    propagation; -metrics=<file> adds JSON lines next to the progress lines,
    whose residual falls as the Anderson iteration converges."""
    import json
    from scft_gb300 import fields
    p = orc.Params(nx=16, ny=16, nz=8, lx=4.0, ly=4.0, lz=2.0, hAB=20.0, fA=0.5, ds0=0.01,
                   batch=1)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=5, batch=1)
    d = str(tmp_path)
    write_case(orc, d, p, wa, wb)
    with open(os.path.join(d, "ab.txt"), "a") as f:
        f.write("mixing=anderson\nhistory=10\nstart=1e9\nprecision=fp32\n")
    r = subprocess.run([DRIVER, "-step=60", "-metrics=m.jsonl"], cwd=d, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    progress = [l for l in r.stdout.splitlines() if l.startswith("GPU ")]
    rows = [json.loads(l) for l in open(os.path.join(d, "m.jsonl")).read().splitlines()]
    assert len(progress) == len(rows) == 6
    for l, row in zip(progress, rows):
        vals = [float(v) for v in l.split(":")[2].split(",")]
        np.testing.assert_allclose(vals, [row[k] for k in ("F", "F_AB", "F_W", "F_S",
                                                            "inCompMax")],
                                   rtol=1e-8, atol=1e-14)
    assert rows[-1]["residual_max"] < 0.1 * rows[0]["residual_max"]
    # the same case with simple mixing (the default without the keys) has not
    # got as far after 60 iterations; were the keys ignored, the runs would agree
    with open(os.path.join(d, "ab.txt")) as f:
        base = "".join(f.readlines()[:7])
    with open(os.path.join(d, "ab.txt"), "w") as f:
        f.write(base + "precision=fp32\n")
    r = subprocess.run([DRIVER, "-step=60", "-metrics=s.jsonl"], cwd=d, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    simple = [json.loads(l) for l in open(os.path.join(d, "s.jsonl")).read().splitlines()]
    assert simple[-1]["residual_max"] > rows[-1]["residual_max"]


def test_driver_double_float(pkg, orc, tmp_path):
    """-precision=df: FP32-pair propagation gives the oracle's progress lines
    to the 9 digits the line prints."""
    from scft_gb300 import fields
    p = orc.Params(nx=64, ny=32, nz=32, lx=4.0, ly=3.0, lz=3.0, hAB=20.0, fA=0.5, ds0=0.02,
                   batch=1)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=6, batch=1)
    d = str(tmp_path)
    write_case(orc, d, p, wa, wb)
    r = subprocess.run([DRIVER, "-step=20", "-precision=df"], cwd=d, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("GPU ")]
    assert len(lines) == 2
    wa0 = orc.read_phi_dat(os.path.join(d, "phi_1.dat"), p.M)[2].reshape((1,) + p.shape)
    wb0 = orc.read_phi_dat(os.path.join(d, "phi_1.dat"), p.M)[3].reshape((1,) + p.shape)
    ref = orc.free_loop(wa0, wb0, p, 20)
    for l, row in zip(lines, ref.log):
        it, b, F, fab, fw, fs, inc = row
        vals = [float(v) for v in l.split(":")[2].split(",")]
        np.testing.assert_allclose(vals[:4], [F, fab, fw, fs], rtol=2e-8, atol=1e-12)


def test_driver_missing_config(pkg, tmp_path):
    r = subprocess.run([DRIVER, "-step=1"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=120)
    assert r.returncode != 0
    assert "ab.txt did not exist" in r.stdout


def test_struct_api_reference_layout(pkg, orc, tmp_path):
    """A driver built with -DSCFT_COMPAT_FP64_LAYOUT sees qa_cu/qcb_cu in the
    reference's g[b][r][s] FP64 layout after getConc (cuda_aid.cu:237)."""
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    pkgdir = os.path.join(ROOT, "scft_ver1.01_gb300")
    exe = str(tmp_path / "layout_check")
    r = subprocess.run([nvcc, "-std=c++17", "-DSCFT_COMPAT_FP64_LAYOUT",
                        "-I" + os.path.join(ROOT, "include", "compat"),
                        "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "native", "compat_layout_check.cpp"),
                        "-L" + pkgdir, "-lscft_gb300", "-Xlinker", "-rpath=" + pkgdir, "-o", exe],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    from scft_gb300 import fields
    p = orc.Params(nx=16, ny=12, nz=8, lx=4.0, ly=3.0, lz=2.0, hAB=20.0, fA=0.4, ds0=0.02,
                   batch=2)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=3, batch=2)
    d = str(tmp_path)
    write_case(orc, d, p, wa, wb)
    r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("layout_maxdiff=")][0]
    assert line == "layout_maxdiff=0 reference_layout=1", line
