"""Generate the config-1 golden fixture: the lamellar 32^3 case solved to
convergence by the CPU oracle.

Config 1 is the plain SCFT case the reference can run on its own: AB diblock
f=0.5, chiN=20, 32^3 periodic grid, box 4.0 Rg per side, Ns=100, FP64, simple
mixing with lambda (wopt) = 0.1, wA/wB = +-chiN*0.1*cos(2 pi x/L) + N(0, 0.01)
from seed 0, run until the max-norm residual of the field update is below
1e-8.  The oracle (oracle/scft_oracle.py, converge_loop) takes about 1300
iterations and a few minutes on the CPU, too long for a test, so this script
stores what a test needs:

  iterations, F (its five parts), Q, the first 20 residual norms, every 50th
  residual norm, phiA/phiB at 4096 seeded points and their moments.

    python tests/golden/make_config1_golden.py [--out tests/golden/config1_lamellar32.npz]
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import scft_oracle as orc  # noqa: E402

GRID, BOX, CHIN, FA, DS0, WOPT, TOL, MAX_IT = 32, 4.0, 20.0, 0.5, 0.01, 0.1, 1e-8, 5000
N_SAMPLES = 4096


def fields_module():
    spec = importlib.util.spec_from_file_location(
        "scft_fields", os.path.join(ROOT, "scft_ver1.01_gb300", "fields.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden", "config1_lamellar32.npz"))
    args = ap.parse_args()
    fl = fields_module()
    wa, wb = fl.lamellar(GRID, GRID, GRID, BOX, BOX, BOX, CHIN, seed=0)
    p = orc.Params(nx=GRID, ny=GRID, nz=GRID, lx=BOX, ly=BOX, lz=BOX, hAB=CHIN, fA=FA, ds0=DS0,
                   wopt=WOPT)
    t0 = time.time()
    ra, rb, pa, pb, Q, iters, errs = orc.converge_loop(wa, wb, p, TOL, MAX_IT, mixing="simple")
    F = orc.free_energy(ra, rb, pa, pb, Q, p.hAB)
    idx = np.random.default_rng(1).choice(p.M, N_SAMPLES, replace=False)
    np.savez_compressed(
        args.out, iterations=iters, F=np.array([f[0] for f in F]), Q=Q, errs_first=np.array(errs[:20]),
        errs_every50=np.array(errs[49::50]), sample_index=idx,
        pha_samples=pa.reshape(-1)[idx], phb_samples=pb.reshape(-1)[idx],
        pha_moments=np.array([pa.mean(), pa.std(), pa.min(), pa.max()]),
        phb_moments=np.array([pb.mean(), pb.std(), pb.min(), pb.max()]))
    print("iterations %d, F %.12f, Q %.12f, %.0f s -> %s" % (iters, F[0][0], Q[0],
                                                           time.time() - t0, args.out))


if __name__ == "__main__":
    main()
