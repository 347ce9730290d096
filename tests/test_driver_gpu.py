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


REF_MAIN_STAGED = os.path.join(ROOT, "oracle", "_ref", "ref_main.cpp")


def build_reference_main(tmp_path):
    """The reference's main.cpp (main.cpp:20-41), unchanged, compiled against
    include/compat/ and linked with this library.  oracle/Makefile stages it
    byte for byte beside the reference-kernel cubin; -I- keeps its quoted
    includes off the directory it sits in."""
    import shutil
    if not os.path.exists(REF_MAIN_STAGED):
        pytest.skip("reference driver source not staged (oracle/_ref/ref_main.cpp)")
    pkgdir = os.path.join(ROOT, "scft_ver1.01_gb300")
    exe = str(tmp_path / "ref_driver")
    r = subprocess.run([shutil.which("g++"), "-std=c++17", "-iquote",
                        os.path.join(ROOT, "include", "compat"), "-I-",
                        "-I" + os.path.join(ROOT, "include", "compat"),
                        "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include",
                        REF_MAIN_STAGED, "-L" + pkgdir, "-lscft_gb300",
                        "-Wl,-rpath=" + pkgdir, "-o", exe],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_main_runs_unchanged(pkg, orc, tmp_path):
    """The reference's own driver gives the same progress lines and pha files
    as this library's driver, and the oracle's Free loop."""
    exe = build_reference_main(tmp_path)
    from scft_gb300 import fields
    p = orc.Params(nx=16, ny=16, nz=8, lx=4.0, ly=4.0, lz=2.0, hAB=20.0, fA=0.5, ds0=0.01,
                   batch=2)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=8, batch=2)
    out = {}
    for name, prog in (("ref", exe), ("ours", DRIVER)):
        d = tmp_path / name
        d.mkdir()
        write_case(orc, str(d), p, wa, wb)
        r = subprocess.run([prog, "-step=100"], cwd=str(d), capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        out[name] = ([l for l in r.stdout.splitlines() if l.startswith("GPU ")],
                     [open(d / ("pha_%d.dat" % (i + 1))).read() for i in range(2)])
        assert any(l.startswith("time=") for l in r.stdout.splitlines())
    assert len(out["ref"][0]) == 20
    assert out["ref"] == out["ours"]                # identical lines and files
    d = str(tmp_path / "ref")
    wa0 = np.stack([orc.read_phi_dat(os.path.join(d, "phi_%d.dat" % (i + 1)), p.M)[2]
                    for i in range(2)]).reshape((2,) + p.shape)
    wb0 = np.stack([orc.read_phi_dat(os.path.join(d, "phi_%d.dat" % (i + 1)), p.M)[3]
                    for i in range(2)]).reshape((2,) + p.shape)
    ref = orc.free_loop(wa0, wb0, p, 100)
    for l, row in zip(out["ref"][0], ref.log):
        it, b, F, fab, fw, fs, inc = row
        assert l.startswith("GPU 0 batch %d: %5d :" % (b, it))
        vals = [float(v) for v in l.split(":")[2].split(",")]
        np.testing.assert_allclose(vals[:4], [F, fab, fw, fs], rtol=1e-7, atol=1e-9)
    pa = orc.read_phi_dat(os.path.join(d, "pha_1.dat"), p.M)[0]
    np.testing.assert_allclose(pa, ref.pha[0].ravel(), rtol=1e-4, atol=1e-5)


def test_driver_splits_instances_over_devices(pkg, orc, tmp_path):
    """-GPU_N=2 with both shards listed on device 0 (the only one a test box
    has): three instances split as the reference does (init_cuda.cu:312,
    batch = 3/2 = 1 per device, the third not run); the progress lines
    number devices and instances as the reference's Free prints them
    (cuda_scft.cu:221) and pha_<g*batch+i+1>.dat holds each shard's instance."""
    from scft_gb300 import fields
    p = orc.Params(nx=16, ny=16, nz=8, lx=4.0, ly=4.0, lz=2.0, hAB=20.0, fA=0.5, ds0=0.01,
                   batch=3)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=9, batch=3)
    d = str(tmp_path)
    write_case(orc, d, p, wa, wb)
    r = subprocess.run([DRIVER, "-step=100", "-GPU_N=2", "-gpu0=0", "-gpu1=0"], cwd=d,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Instances 3 to 3 are not run" in r.stdout
    lines = [l for l in r.stdout.splitlines() if l.startswith("GPU ")]
    assert len(lines) == 20                      # every 10 iterations x 2 shards x 1 instance
    assert lines[0].startswith("GPU 0 batch 0:") and lines[1].startswith("GPU 1 batch 0:")
    assert not os.path.exists(os.path.join(d, "pha_3.dat"))
    p1 = orc.Params(nx=16, ny=16, nz=8, lx=4.0, ly=4.0, lz=2.0, hAB=20.0, fA=0.5, ds0=0.01,
                    batch=1)
    for g in range(2):
        fn = os.path.join(d, "phi_%d.dat" % (g + 1))
        w = orc.read_phi_dat(fn, p.M)
        ref = orc.free_loop(w[2].reshape((1,) + p.shape), w[3].reshape((1,) + p.shape), p1, 100)
        mine = [l for l in lines if l.startswith("GPU %d batch 0:" % g)]
        for l, row in zip(mine, ref.log):
            vals = [float(v) for v in l.split(":")[2].split(",")]
            np.testing.assert_allclose(vals[:4], row[2:6], rtol=1e-7, atol=1e-9)
        pa = orc.read_phi_dat(os.path.join(d, "pha_%d.dat" % (g + 1)), p.M)[0]
        np.testing.assert_allclose(pa, ref.pha[0].ravel(), rtol=1e-4, atol=1e-5)


def test_driver_refuses_a_missing_device(pkg, orc, tmp_path):
    import torch
    from scft_gb300 import fields
    p = orc.Params(nx=16, ny=16, nz=8, lx=4.0, ly=4.0, lz=2.0, hAB=20.0, fA=0.5, ds0=0.01,
                   batch=2)
    wa, wb = fields.lamellar(p.nx, p.ny, p.nz, p.lx, p.ly, p.lz, 20.0, seed=9, batch=2)
    d = str(tmp_path)
    write_case(orc, d, p, wa, wb)
    missing = torch.cuda.device_count()
    r = subprocess.run([DRIVER, "-step=10", "-GPU_N=2", "-gpu1=%d" % missing], cwd=d,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "-gpu1=%d names no device" % missing in r.stderr
