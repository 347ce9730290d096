"""Pin the VTK writer to the reference converter's own output.

The reference ships out.vtk, the output of its converter (vtk.c) on a 106x106x1
pha_1.dat.  This script, run where the reference tree is readable, records
what the test needs to rebuild and compare that file byte for byte: the header
values, the 11236 printed values (as integers in units of 1e-4) and the
SHA-256 of the whole file.

    python tests/golden/make_vtk_golden.py [REFERENCE_DIR]
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    raw = open(os.path.join(ref, "out.vtk"), "rb").read()
    lines = raw.decode().split("\n")
    source = lines[1].split("converted from file ")[1]
    nx, ny, nz = (int(t) for t in lines[4].split()[1:])
    spacing = np.array([float(t) for t in lines[6].split()[1:]])
    rows = lines[12:12 + ny * nz]
    vals = np.array([float(t) for r in rows for t in r.split()])
    assert vals.size == nx * ny * nz
    ival = np.rint(vals * 1e4).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_out_vtk.npz"), source=source,
                        dims=np.array([nx, ny, nz]), spacing=spacing, ival=ival,
                        sha256=hashlib.sha256(raw).hexdigest(), size=len(raw))
    print("wrote ref_out_vtk.npz", nx, ny, nz, spacing, len(raw))


if __name__ == "__main__":
    main()
