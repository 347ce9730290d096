"""Generate the golden vectors that pin the CPU oracle to the reference.

Runs on a GPU machine: the reference's own kernels (compiled unchanged from the
reference sources into oracle/_ref/ref_kernels.cubin by oracle/Makefile) are
driven by oracle/ref_harness.cpp in the reference's host order with cuFFT.
For each case the seeded input fields and the reference outputs are written
to tests/golden/ref_<case>.npz (or --out DIR).  tests/test_ref_golden.py then
checks the oracle against them on the CPU.

Q: the reference's cal_ql kernel (cuda_aid.cu:119-168) writes each thread's
partial sum to shared memory and starts the tree reduction without a barrier,
so on GB300 it returns a corrupted sum.  The harness therefore takes Q from the
FP64 sum of the reference's own qB[.][dNsB] slice (q_mode 1) and records the
kernel's raw value beside it (calql_raw, calql_repeat).

    python tests/golden/make_ref_golden.py [--out DIR] [--time]

--time also prints the reference's own GPU time per SCF iteration at the
128^3, Ns=200 benchmark workload (one JSON line).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

# (name, grid, box, chiN, fA, ds0, batch, init, iterations)
CASES = [
    ("lam16", (16, 16, 16), (4.0, 4.0, 4.0), 20.0, 0.5, 0.01, 2, "lamellar", 20),
    ("gyr32x16x8", (32, 16, 8), (3.8, 3.8, 3.8), 18.0, 0.36, 0.02, 1, "gyroid", 10),
    ("film32x32x1", (32, 32, 1), (4.0, 4.0, 2.0), 20.0, 0.5, 0.01, 1, "lamellar", 10),
    ("radix3_24x16x8", (24, 16, 8), (3.0, 3.2, 2.4), 15.0, 0.4, 0.025, 2, "random", 5),
    ("hex32x16x8", (32, 16, 8), (4.2, 7.2746, 2.0), 25.0, 0.3, 0.02, 1, "hexagonal", 5),
]
# 12^3: the reference's reduction thread count (largest divisor of M <= 1024)
# is 864, not a power of two, so reduce3 drops terms; only average_value is
# recorded for this case.
QUIRK_CASE = ("quirk12", (12, 12, 12), (3.0, 3.0, 3.0))


def fields_for(init, grid, box, chiN, seed, batch):
    import __graft_entry__ as ge
    ge.load_package()
    from scft_gb300 import fields as fl
    nx, ny, nz = grid
    lx, ly, lz = box
    if init == "lamellar":
        return fl.lamellar(nx, ny, nz, lx, ly, lz, chiN, seed, batch)
    if init == "gyroid":
        return fl.gyroid(nx, ny, nz, lx, ly, lz, chiN, seed, batch)
    if init == "hexagonal":
        return fl.hexagonal(nx, ny, nz, lx, ly, lz, chiN, seed, batch)
    return fl.random_fields(nx, ny, nz, seed, batch, scale=1.5)


def run_case(case, outdir):
    from oracle.ref_harness import RefSolver
    name, grid, box, chiN, fA, ds0, batch, init, iters = case
    wa, wb = fields_for(init, grid, box, chiN, 7, batch)
    r = RefSolver(*grid, *box, chiN, fA, ds0, batch)
    r.set_w(wa, wb)
    r.get_conc()
    out = dict(grid=np.array(grid), box=np.array(box), chiN=chiN, fA=fA, ds0=ds0, batch=batch,
               wa_in=wa, wb_in=wb, conc_wa=r.get_field(0), conc_pha=r.get_field(2),
               conc_phb=r.get_field(3), conc_Q=r.Q(),
               qa_end=r.get_q(0, r.NsA), qcb_0=r.get_q(1, 0), qb_end=r.get_q(2, r.dNsB),
               qca_0=r.get_q(3, 0), qca_mid=r.get_q(3, r.NsA // 2),
               # the reference's cal_ql kernel value of that getConc, and five
               # back-to-back re-runs of it on the same slice (its shared-memory race)
               calql_raw=r.ql_raw(), calql_repeat=r.cal_ql_repeat(5))
    r.set_w(wa, wb)
    fe = r.iterate(iters)
    out.update(iters=iters, loop_wa=r.get_field(0), loop_wb=r.get_field(1),
               loop_pha=r.get_field(2), loop_phb=r.get_field(3), loop_Q=r.Q(), loop_fe=fe)
    r.close()
    path = os.path.join(outdir, f"ref_{name}.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


def run_quirk(outdir):
    from oracle.ref_harness import RefSolver
    name, grid, box = QUIRK_CASE
    rng = np.random.default_rng(11)
    w = rng.normal(0.3, 1.0, (1,) + grid[::-1])
    r = RefSolver(*grid, *box, 15.0, 0.5, 0.05, 1)
    r.set_w(w, w)
    r.average_value(0)
    np.savez_compressed(os.path.join(outdir, f"ref_{name}.npz"), grid=np.array(grid), w_in=w,
                        w_avg=r.get_field(0))
    r.close()


def run_constrained(outdir):
    """phi_w_constrained (lambda 0.7) and phi_w_constrainedEx
    (cuda_aid.cu:418-490) of the reference on seeded fields, batch 2."""
    from oracle.ref_harness import RefSolver
    grid, box, chiN, lam = (16, 12, 8), (3.0, 3.0, 2.0), 17.0, 0.7
    rng = np.random.default_rng(23)
    shape = (2,) + grid[::-1]
    wa = rng.normal(0.0, 2.0, shape)
    wb = rng.normal(0.0, 2.0, shape)
    pha = rng.uniform(0.05, 0.95, shape)
    phb = 1.0 - pha + rng.normal(0.0, 0.02, shape)
    target = rng.uniform(0.0, 1.0, shape)
    out = dict(grid=np.array(grid), box=np.array(box), chiN=chiN, lam=lam, wa_in=wa, wb_in=wb,
               pha=pha, phb=phb, target=target)
    r = RefSolver(*grid, *box, chiN, 0.5, 0.05, 2)
    for key, ex in (("con", False), ("conex", True)):
        r.set_w(wa, wb)
        r.set_field(2, pha)
        r.set_field(3, phb)
        r.set_target(target)
        r.phi_w_constrained(ex, lam)
        out[key + "_wa"] = r.get_field(0)
        out[key + "_wb"] = r.get_field(1)
    r.close()
    path = os.path.join(outdir, "ref_constrained16x12x8.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


def time_reference():
    from oracle.ref_harness import RefSolver
    n, L = 128, 3.8
    wa, wb = fields_for("gyroid", (n, n, n), (L, L, L), 18.0, 0, 1)
    r = RefSolver(n, n, n, L, L, L, 18.0, 0.36, 0.005, 1)
    r.set_q_mode(0)        # time the reference exactly as it runs (cal_ql kernel)
    r.set_w(wa, wb)
    r.iterate(1, with_energy=False)          # warm-up (plans, modules)
    ms = r.time_iterations(2) / 2
    pts = 2 * (r.NsA + r.dNsB) * n ** 3
    r.close()
    print(json.dumps({"reference_gpu": {"workload": "128^3 gyroid, Ns=200, 1 SCF iteration",
                                        "ms_per_iteration": ms,
                                        "gpt_step_per_s": pts / (ms / 1e3) / 1e9,
                                        "arith": "fp64 (reference kernels + cuFFT D2Z/Z2D)"}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    ap.add_argument("--time", action="store_true")
    ap.add_argument("--only", nargs="*", default=None,
                    help="case names to (re)generate (default: all); 'quirk12', 'constrained'")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    want = lambda n: args.only is None or n in args.only
    for c in CASES:
        if want(c[0]):
            run_case(c, args.out)
    if want("quirk12"):
        run_quirk(args.out)
    if want("constrained"):
        run_constrained(args.out)
    if args.time:
        time_reference()


if __name__ == "__main__":
    main()
