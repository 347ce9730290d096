"""VTK export pinned to the reference converter's own output file (vtk.c ->
out.vtk, 106x106x1): the oracle's formatter and the C-ABI converter both
rebuild it byte for byte from its values.  Host-only code: no GPU needed."""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_out_vtk.npz")


@pytest.fixture(scope="module")
def gold():
    g = np.load(GOLD)
    return dict(source=str(g["source"]), dims=tuple(int(v) for v in g["dims"]),
                spacing=tuple(float(v) for v in g["spacing"]), vals=g["ival"] / 1e4,
                sha=str(g["sha256"]), size=int(g["size"]))


def write_pha(path, dims, spacing, pa1, pa2):
    nx, ny, nz = dims
    with open(path, "w") as f:
        f.write("Nx=%d, Ny=%d, Nz=%d\n" % dims)
        f.write("dx=%g, dy=%g, dz=%g\n" % spacing)
        for a, b in zip(pa1, pa2):
            f.write("%g %g 0 0\n" % (a, b))


def test_oracle_vtk_text_matches_reference_file(orc, gold):
    text = orc.vtk_text(gold["source"], *gold["dims"], *gold["spacing"], gold["vals"])
    raw = text.encode()
    assert len(raw) == gold["size"]
    assert hashlib.sha256(raw).hexdigest() == gold["sha"]


def test_capi_converter_matches_reference_file(pkg, gold, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    v = gold["vals"]
    # phiA - phiB split into two columns so the subtraction is exercised
    pa2 = np.round(np.linspace(0.0, 0.3, v.size), 4)
    pa1 = np.round(v + pa2, 4)
    assert np.array_equal(np.round(pa1 - pa2, 4), v)
    write_pha(gold["source"], gold["dims"], gold["spacing"], pa1, pa2)
    pkg.convert_pha_to_vtk(gold["source"], "out.vtk")
    raw = open("out.vtk", "rb").read()
    assert len(raw) == gold["size"]
    assert hashlib.sha256(raw).hexdigest() == gold["sha"]
    assert orc_text_equal(raw, gold["source"])


def orc_text_equal(raw, source):
    from oracle import scft_oracle
    return raw.decode() == scft_oracle.convert_pha_to_vtk(source)


def test_converter_reports_missing_and_short_files(pkg, tmp_path):
    with pytest.raises(pkg.ScftError):
        pkg.convert_pha_to_vtk(str(tmp_path / "absent.dat"), str(tmp_path / "o.vtk"))
    p = tmp_path / "short.dat"
    p.write_text("Nx=4, Ny=2, Nz=1\ndx=0.5, dy=0.5, dz=1\n0.1 0.2 0 0\n")
    with pytest.raises(pkg.ScftError):
        pkg.convert_pha_to_vtk(str(p), str(tmp_path / "o.vtk"))
