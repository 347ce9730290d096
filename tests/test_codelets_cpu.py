"""The in-register DFT codelets of the fast kernels (csrc/fft_reg.cuh) are
host+device code; compile them for the host and check every size the
kernels instantiate against a naive long-double DFT (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_codelets_match_naive_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "codelet_check")
    src = os.path.join(ROOT, "tests", "native", "codelet_check.cu")
    inc = os.path.join(ROOT, "scft_ver1.01_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-I" + inc, "-o", exe, src],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
