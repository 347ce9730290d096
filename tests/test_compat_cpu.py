"""Host-side pieces of the struct API and its device split, without a GPU:
the reference's split of Num_SCFT instances over GPU_N devices
(init_cuda.cu:312), the -GPU_N / -gpu<i> device map (init.cpp:20-35), and the
reference's own driver main.cpp compiled unchanged against include/compat/."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKGDIR = os.path.join(ROOT, "scft_ver1.01_gb300")
REF_MAIN = "/root/reference/main.cpp"


@pytest.mark.parametrize("num,gpus,per,not_run", [
    (8, 4, 2, 0), (5, 2, 2, 1), (7, 3, 2, 1), (3, 3, 1, 0), (64, 8, 8, 0), (65, 8, 8, 1),
    (1, 1, 1, 0)])
def test_shard_plan_matches_the_reference_split(pkg, num, gpus, per, not_run):
    """batch = Num_SCFT / GPU_N per device; the remainder is not run."""
    assert pkg.shard_plan(num, gpus) == (per, not_run)
    assert per == num // gpus and not_run == num - per * gpus


@pytest.mark.parametrize("num,gpus", [(2, 3), (0, 1), (4, 0), (100, 65)])
def test_shard_plan_refuses_empty_shards(pkg, num, gpus):
    with pytest.raises(pkg.ScftError) as e:
        pkg.shard_plan(num, gpus)
    assert e.value.status == pkg.ERR_INVALID_ARG


def compile_cpp(src, exe, extra=()):
    gxx = shutil.which("g++")
    cmd = [gxx, "-std=c++17", *extra, "-I" + os.path.join(ROOT, "include", "compat"),
           "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include", src,
           "-L" + PKGDIR, "-lscft_gb300", "-Wl,-rpath=" + PKGDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("args,want", [
    ([], "GPU_N=1 map=0"),
    (["-GPU_N=3", "-gpu0=2", "-gpu1=0", "-gpu2=1"], "GPU_N=3 map=2,0,1"),
    (["-GPU_N=2", "-gpu1=5"], "GPU_N=2 map=0,5"),      # an unlisted index maps to device 0
])
def test_device_map_flags(pkg, tmp_path, args, want):
    exe = compile_cpp(os.path.join(ROOT, "tests", "native", "compat_flags_check.cpp"),
                      str(tmp_path / "flags_check"))
    r = subprocess.run([exe, "-kernal=CPU", "-step=7"] + args, cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("kernal_type=")][0]
    assert line == f"kernal_type=2 {want} MaxIT=7", line


@pytest.mark.skipif(not os.path.exists(REF_MAIN), reason="reference sources absent")
def test_reference_main_compiles_and_links_unchanged(pkg, tmp_path):
    """The reference's main.cpp, compiled from where it lies: -I- stops the
    quoted includes from resolving to the reference's own headers beside it,
    so struct.h, init.h, init_cuda.h and cuda_scft.h are the compat ones."""
    exe = compile_cpp(REF_MAIN, str(tmp_path / "ref_driver"),
                      extra=("-iquote", os.path.join(ROOT, "include", "compat"), "-I-"))
    # the CPU branch (no device needed): the reference's messages, and its
    # unconditional fft_test call on an uninitialised solver is harmless
    r = subprocess.run([exe, "-kernal=CPU"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "In this programm, we use CPU." in r.stdout
    assert "fft_test did not successfully detect run time" in r.stdout
