"""The C-ABI library builds, loads and exports every declared symbol; host
logic that needs no GPU (parameters, grid support, ab.txt parsing, error
paths).  No compute call is made here."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(scft_\w+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(pkg):
    lib = C.CDLL(pkg.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert names == set(pkg.EXPORTS)


def test_params_default_matches_reference_constants(pkg):
    p = pkg.default_params()
    assert (p.nx, p.ny, p.nz, p.batch) == (32, 32, 32, 1)
    assert (p.wopt, p.wcmp) == (0.05, 0.10)     # cuda_aid.cu:395-396
    assert p.precision == pkg.PREC_FP64 and p.mixing == pkg.MIX_SIMPLE


def test_grid_supported(pkg):
    lib = pkg.load_library()
    assert lib.scft_grid_supported(32, 32, 32)
    assert lib.scft_grid_supported(128, 128, 64)
    assert lib.scft_grid_supported(48, 48, 48)
    assert lib.scft_grid_supported(480, 480, 1)
    assert lib.scft_grid_supported(106, 106, 1)      # 2*53: generic radix
    assert lib.scft_grid_supported(24, 20, 18)
    assert not lib.scft_grid_supported(33, 32, 32)   # odd Nx
    assert not lib.scft_grid_supported(32, 31, 32)   # odd Ny > 1
    assert not lib.scft_grid_supported(1, 32, 32)    # Nx = 1
    assert not lib.scft_grid_supported(2 * 67, 8, 8)  # prime factor > 61


def test_strerror(pkg):
    lib = pkg.load_library()
    assert lib.scft_strerror(0) == b"ok"
    assert lib.scft_strerror(pkg.ERR_UNSUPPORTED).startswith(b"unsupported")


def test_create_rejects_bad_params_without_gpu(pkg):
    # argument validation happens before any device call
    with pytest.raises(pkg.ScftError) as e:
        pkg.Context(nx=33)
    assert e.value.status == pkg.ERR_UNSUPPORTED
    with pytest.raises(pkg.ScftError) as e:
        pkg.Context(ds0=-1.0)
    assert e.value.status == pkg.ERR_INVALID_ARG
    with pytest.raises(pkg.ScftError) as e:
        pkg.Context(precision=7)
    assert e.value.status == pkg.ERR_INVALID_ARG


def test_read_ab_txt(pkg, tmp_path):
    f = tmp_path / "ab.txt"
    f.write_text("intag=1024\nxN=25.0\nfa=0.300\nlx=4.2, ly=7.2746, lz=2.0\n"
                 "Nx=128, Ny=128, Nz=64\nds0=0.005\nbatch=3\n")
    p, tag = pkg.read_ab_txt(str(f))
    assert tag == 1024
    assert (p.nx, p.ny, p.nz, p.batch) == (128, 128, 64, 3)
    assert (p.hAB, p.fA, p.ds0) == (25.0, 0.3, 0.005)
    assert (p.lx, p.ly, p.lz) == (4.2, 7.2746, 2.0)


def test_read_ab_txt_errors(pkg, tmp_path):
    with pytest.raises(pkg.ScftError) as e:
        pkg.read_ab_txt(str(tmp_path / "missing.txt"))
    assert e.value.status == pkg.ERR_IO
    f = tmp_path / "ab.txt"
    f.write_text("intag=1024\nxN=oops\n")
    with pytest.raises(pkg.ScftError) as e:
        pkg.read_ab_txt(str(f))
    assert e.value.status == pkg.ERR_IO


AB7 = ("intag=1024\nxN=25.0\nfa=0.300\nlx=4.2, ly=7.2746, lz=2.0\n"
       "Nx=128, Ny=128, Nz=64\nds0=0.005\nbatch=3\n")


def test_read_ab_txt_optional_keys(pkg, tmp_path):
    f = tmp_path / "ab.txt"
    f.write_text(AB7 + "# solver options\nmixing=anderson\nhistory=30\nlambda=0.4\nstart=0.5\n"
                 "wopt=0.02\nwcmp=0.2\nprecision=fp32\nNs=400\n\n")
    p, tag = pkg.read_ab_txt(str(f))
    assert tag == 1024 and (p.nx, p.nz, p.batch) == (128, 64, 3)
    assert p.mixing == pkg.MIX_ANDERSON and p.anderson_history == 30
    assert (p.anderson_lambda, p.anderson_start, p.wopt, p.wcmp) == (0.4, 0.5, 0.02, 0.2)
    assert p.precision == pkg.PREC_FP32 and p.ds0 == 1.0 / 400
    f.write_text(AB7 + "precision=df\n")
    assert pkg.read_ab_txt(str(f))[0].precision == pkg.PREC_DF
    # without the optional lines: the reference's defaults
    f.write_text(AB7)
    p, _ = pkg.read_ab_txt(str(f))
    assert p.mixing == pkg.MIX_SIMPLE and p.precision == pkg.PREC_FP64
    assert (p.wopt, p.wcmp, p.ds0) == (0.05, 0.10, 0.005)


@pytest.mark.parametrize("extra", ["mixing=broyden\n", "history=lots\n", "colour=blue\n",
                                   "just text\n", "Ns=0\n"])
def test_read_ab_txt_rejects_bad_optional_keys(pkg, tmp_path, extra):
    f = tmp_path / "ab.txt"
    f.write_text(AB7 + extra)
    with pytest.raises(pkg.ScftError) as e:
        pkg.read_ab_txt(str(f))
    assert e.value.status == pkg.ERR_IO


def test_params_layout_matches_header(pkg, tmp_path):
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "scft_capi.h"\n'
                   'int main(void){printf("%zu %zu %zu\\n", sizeof(scft_params),'
                   ' offsetof(scft_params, anderson_start), offsetof(scft_params, flags));'
                   'return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    size, off_start, off_flags = map(int, subprocess.run([str(exe)], capture_output=True,
                                                          text=True).stdout.split())
    assert C.sizeof(pkg.ScftParams) == size
    assert pkg.ScftParams.anderson_start.offset == off_start
    assert pkg.ScftParams.flags.offset == off_flags


def test_library_refuses_to_load_when_missing(pkg, tmp_path):
    with pytest.raises(ImportError):
        pkg.load_library(str(tmp_path / "nope.so"))
