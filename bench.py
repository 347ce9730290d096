"""Benchmark of the SCFT propagator hot path on GB300.

Metric: Gpt*step/s (grid points x contour steps per second) at 128^3, Ns=200,
reported with the HBM-roofline fraction of the propagator march.

One "step" = one SCF iteration of the reference's Free loop
(cuda_scft.cu:167-186): average_value x3, four propagator marches
(2*(NsA+dNsB) contour steps over M points), Q, phi and the field update.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 runs under torchrun: every rank solves its own independent replica (the
path has no exchange step), and rank 0 prints the whole-job rate computed
from the max-over-ranks time.  --impl reference times the reference's
algorithm on the host cores (the reference has no CPU path of its own, so
this is the CPU restatement with threaded scipy.fft) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpt·step/s at 128³ Ns=200 (%HBM roofline); s-to-converge vs plain FP64 GPU"
UNIT = "Gpt*step/s"
N, L, CHIN, FA, DS = 128, 3.8, 18.0, 0.36, 0.005
WORKLOAD = ("128^3 periodic grid, double-gyroid init chiN*0.2*g(r)+N(0,0.02) seed 0, "
            "f=0.36, chiN=18, box 3.8 Rg, Ns=200 (ds=0.005, NsA=72, dNsB=128), "
            "1 SCF iteration (4 propagator marches + Q + phi + simple mixing) per step")
BYTES_PER_PT_STEP = {"fp32": 12.0, "fp64": 24.0, "df": 24.0}
# DRAM bytes (read + write) of one march launch = one contour step of one
# propagator at 128^3 FP32, from an ncu capture with warm L2 (--cache-control
# none): the slice's write-back only, against 25.2 MB of algorithmic bytes --
# the other operands stay in L2.
TRAFFIC_PER_STEP = 8.48e6
TRAFFIC_NOTE = ("dram bytes per launch (one contour step) with warm L2, mean of 4 launches of "
                "k_xyxy/k_zz from one ncu capture of the Ns=20 case; algorithmic bytes per "
                "launch: 12 B x 128^3 = 25.2 MB")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, dist, device):
    """The largest x over all ranks (the job's time is its slowest rank's)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    smax.append(float(parts[1]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[4:8]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(seconds=10.0):
    """The CPU restatement (scipy.fft, all host threads) on a bounded sample of
    the same workload: full SCF iterations of the 128^3 gyroid (one untimed,
    then as many as fit in about `seconds`, at least two)."""
    from oracle import scft_oracle as orc
    import __graft_entry__ as ge
    ge.load_package()
    from scft_gb300 import fields as fl
    p = orc.Params(nx=N, ny=N, nz=N, lx=L, ly=L, lz=L, hAB=CHIN, fA=FA, ds0=DS)
    wa, wb = fl.gyroid(N, N, N, L, L, L, CHIN, seed=0)
    workers = os.cpu_count()
    wa, wb, *_ = orc.iteration_cpu(wa, wb, p, workers)   # warm-up (plans, pages)
    done_s, its = 0.0, 0
    while done_s < seconds or its < 2:
        t0 = time.perf_counter()
        wa, wb, *_ = orc.iteration_cpu(wa, wb, p, workers)
        done_s += time.perf_counter() - t0
        its += 1
    value = its * orc.pt_steps_per_iteration(p) / done_s / 1e9
    return {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{its} full SCF iterations at 128^3, Ns=200 (scipy.fft pocketfft, FP64, "
                      f"{workers} threads), {done_s:.1f} s"}


def reference_cuda_leg(iters=2):
    """The reference's own CUDA build on this GPU: its kernels (cuda_aid.cu,
    compiled unchanged for sm_103a into oracle/_ref/ref_kernels.cubin) driven
    in its host order with cuFFT D2Z/Z2D in FP64 (oracle/ref_harness.cpp), on
    the benchmark workload; timed as its fft_test times Free
    (cuda_scft.cu:411-425): events around whole SCF iterations."""
    try:
        from oracle import ref_harness
        if not ref_harness.available():
            return {"unavailable": "oracle/_ref (the reference kernels + harness) not built"}
        import __graft_entry__ as ge
        ge.load_package()
        from scft_gb300 import fields as fl
        wa, wb = fl.gyroid(N, N, N, L, L, L, CHIN, seed=0)
        r = ref_harness.RefSolver(N, N, N, L, L, L, CHIN, FA, DS, 1)
        r.set_q_mode(0)           # exactly as it runs (its cal_ql kernel)
        r.set_w(wa, wb)
        r.iterate(1, with_energy=False)        # warm-up: plans, module load
        ms = r.time_iterations(iters) / iters
        pts = 2 * (r.NsA + r.dNsB) * N ** 3
        r.close()
        return {"what": "the reference's kernels (unchanged, sm_103a) + cuFFT FP64 in its host "
                        "order, one GB300, 128^3 gyroid Ns=200, CUDA events around %d SCF "
                        "iterations" % iters,
                "ms_per_iteration": ms, "value": pts / (ms / 1e3) / 1e9, "unit": UNIT,
                "dtype": "f64"}
    except Exception as e:                     # no GPU or harness failure: say so
        return {"unavailable": str(e).splitlines()[0][:200]}


def run_reference(args):
    """The reference arm: the reference has no CPU path (init.cpp:119-125), so
    its algorithm runs as the CPU restatement (the oracle, scipy.fft on every
    host thread) on this arm's own workload: one full SCF iteration of the
    128^3 gyroid per step (average_value x2, the four marches, Q, phi, simple
    mixing; cuda_scft.cu:167-253)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import scft_oracle as orc
    import __graft_entry__ as ge
    ge.load_package()
    from scft_gb300 import fields as fl
    p = orc.Params(nx=N, ny=N, nz=N, lx=L, ly=L, lz=L, hAB=CHIN, fA=FA, ds0=DS)
    wa, wb = fl.gyroid(N, N, N, L, L, L, CHIN, seed=0)
    workers = os.cpu_count()
    pts = orc.pt_steps_per_iteration(p)
    for _ in range(args.warmup):
        wa, wb, *_ = orc.iteration_cpu(wa, wb, p, workers)
    tot = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        wa, wb, *_ = orc.iteration_cpu(wa, wb, p, workers)
        tot += time.perf_counter() - t0
    value = pts * args.steps / tot / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [N, N, N], "Ns": 200, "same_config": True},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": f"{args.steps} full SCF iterations at 128^3, Ns=200 (4 "
                                   f"marches + Q + phi + simple mixing); the reference has no "
                                   f"CPU path (init.cpp:119-125), so its algorithm runs as the "
                                   f"CPU restatement with scipy.fft on {workers} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda": reference_cuda_leg() if not args.no_ref_cuda else None,
    }
    print(json.dumps(line), flush=True)
    return 0


def converge_timed(ctx, tol, max_it, budget_s):
    """ctx.converge in chunks of 50 iterations (the Anderson history carries
    over) until converged, max_it, or the wall-clock budget is spent."""
    total, fe = 0, None
    t0 = time.perf_counter()
    while total < max_it:
        it, fe = ctx.converge(tol, min(50, max_it - total))
        total += it
        if float(ctx.residual()[0].max()) < tol:
            return total, fe, True
        if time.perf_counter() - t0 > budget_s:
            break
    return total, fe, False


def converge_until_floor(ctx, tol, max_it, budget_s, chunk=10, patience=40):
    """The FP32 phase of a mixed solve: iterate until the residual is below
    tol, or it has stopped falling (no new minimum below 0.8x the best for
    `patience` iterations: FP32 propagation's round-off floor, which rises
    with the grid: ~2e-5 at 64^3, near 3e-5 at 128^3), or max_it / the
    budget is spent.  Returns the iterations run."""
    total, best, since = 0, float("inf"), 0
    t0 = time.perf_counter()
    while total < max_it:
        it, _ = ctx.converge(tol, min(chunk, max_it - total))
        total += it
        r = float(ctx.residual()[0].max())
        if r < tol:
            break
        if r < 0.8 * best:
            best, since = r, 0
        else:
            since += it
            if since >= patience:
                break
        if time.perf_counter() - t0 > budget_s:
            break
    return total


def translation_aligned_diff(a, b, iters=4):
    """max|a(r) - b(r - d)| / max|a| for the rigid shift d (in voxels, per
    axis) that best aligns b with a, found by Gauss-Newton on the spectral
    shift b(r - d) = IFFT[B(k) exp(-i k.d)].  A converged periodic structure
    is only defined up to such a shift (the translational zero mode), so two
    runs that reach the same structure may differ by it at the same F.
    Returns (relative difference, d)."""
    shape = a.shape
    axes = tuple(range(a.ndim))
    B = np.fft.rfftn(b)
    ks = []
    for ax, n in enumerate(shape):
        f = np.fft.rfftfreq(n) if ax == len(shape) - 1 else np.fft.fftfreq(n)
        k = 2 * np.pi * f
        if n % 2 == 0:
            k[n // 2 if ax < len(shape) - 1 else -1] = 0.0   # no derivative at Nyquist
        sh = [1] * len(shape)
        sh[ax] = k.size
        ks.append(k.reshape(sh))
    d = np.zeros(len(shape))
    for _ in range(iters):
        ph = np.exp(-1j * sum(k * dj for k, dj in zip(ks, d)))
        s = np.fft.irfftn(B * ph, s=shape, axes=axes)
        G = np.stack([np.fft.irfftn(-1j * k * B * ph, s=shape, axes=axes).ravel() for k in ks],
                     axis=1)
        r = (a - s).ravel()
        step = np.linalg.lstsq(G, -r, rcond=None)[0]
        d = d - step
    s = np.fft.irfftn(B * np.exp(-1j * sum(k * dj for k, dj in zip(ks, d))), s=shape, axes=axes)
    return float(np.abs(a - s).max() / np.abs(a).max()), [float(x) for x in d]


def compare_to_fp64(ref, run):
    """Agreement of a converged run with the plain FP64 run: each is
    (phiA, phiB, Q, F) of its last getConc."""
    spec = lambda a: np.abs(np.fft.rfftn(a))
    al, shift = translation_aligned_diff(ref[0][0], run[0][0])
    alb, _ = translation_aligned_diff(ref[1][0], run[1][0])
    return {"F_abs_diff": float(abs(run[3] - ref[3])),
            "Q_rel_diff": float(abs(run[2][0] - ref[2][0]) / abs(ref[2][0])),
            "phiA_rel_diff": float(np.abs(run[0] - ref[0]).max() / np.abs(ref[0]).max()),
            # a converged structure may sit shifted by a fraction of a voxel
            # at the same F (the translational zero mode): compare the moduli
            # of the Fourier coefficients, and pointwise after removing the
            # rigid shift
            "phiA_spectrum_rel_diff": float(np.abs(spec(run[0][0]) - spec(ref[0][0])).max()
                                            / spec(ref[0][0]).max()),
            "phiA_rel_diff_shift_aligned": al, "phiB_rel_diff_shift_aligned": alb,
            "phiA_shift_voxels": shift}


def converge_leg(pkg, dev, n=64, tol=1e-6, max_it=3000, budget_s=150.0, polishes=None,
                 pin=False):
    """Seconds to converge (max-norm residual < tol) on the n^3 double-gyroid
    config (f=0.36, chiN=18, box 3.8, Ns=200, Anderson history 20; n = 64 is
    config 2, n = 128 the metric's own grid): the plain FP64 GPU path against
    FP32 propagation followed by a polish in FP64, and followed by a polish in
    double-float (FP32-pair) arithmetic.  Wall-clock seconds with a residual
    check after every iteration, inputs already on the device.  Each run then
    continues to 1e-7, timed as well: at 1e-6 each run's phi sits within about
    1e-6 of the saddle point, so phi is compared pointwise at 1e-7 too.  pin: every path with SCFT_FLAG_PIN_TRANSLATION (Anderson
    updates without their rigid-shift component), so that the runs reach the
    same unshifted structure and phi is compared pointwise as it stands."""
    from scft_gb300 import fields as fl
    Lb = 3.8
    polishes = polishes or (("fp32_fp64_polish", "fp64"), ("fp32_df_polish", "df"))
    clocks = ClockSampler(dev)   # the leg's clocks: its seconds are wall-clock
    wa, wb = fl.gyroid(n, n, n, Lb, Lb, Lb, 18.0, seed=0)
    # Anderson from the first iteration for every path (measured on this
    # config: FP64 142 iterations against 159 with simple mixing down to 1.0)
    kw = dict(nx=n, ny=n, nz=n, lx=Lb, ly=Lb, lz=Lb, hAB=18.0, fA=0.36, ds0=0.005,
              mixing=pkg.MIX_ANDERSON, anderson_history=20, anderson_lambda=0.5,
              anderson_start=1e9, device=dev, flags=pkg.FLAG_PIN_TRANSLATION if pin else 0)
    out = {"config": "%d^3 double gyroid, f=0.36, chiN=18, box 3.8 Rg, Ns=200, Anderson m=20 "
                     "from the first iteration (every path), tol %g (max-norm of the phi_w "
                     "residual)%s" % (n, tol, ", rigid shifts pinned in every path" if pin
                                      else "")}
    state = lambda c, fe: (c.pha, c.phb, c.Q(), fe[0, 0])

    with pkg.Context(precision=pkg.PREC_FP64, **kw) as c64:
        c64.set_w(wa, wb)
        c64.iterate(1)                      # plans, graph capture
        c64.set_w(wa, wb)
        t0 = time.perf_counter()
        it64, fe64, ok64 = converge_timed(c64, tol, max_it, budget_s)
        t64 = time.perf_counter() - t0
        r64 = float(c64.residual()[0][0])
        ref = state(c64, fe64)
        t0 = time.perf_counter()
        it7, fe, ok = converge_timed(c64, 1e-7, 1000, 40.0)
        t64_7 = t64 + time.perf_counter() - t0
        ref_t = state(c64, fe) if ok else None
    out["fp64"] = {"seconds": t64, "iterations": it64, "F": fe64[0, 0], "residual": r64,
                   "converged": ok64, "seconds_to_1e-7": t64_7, "iterations_to_1e-7": it64 + it7}

    with pkg.Context(precision=pkg.PREC_FP32, **kw) as c32, \
            pkg.Context(precision=pkg.PREC_FP64, **kw) as p64, \
            pkg.Context(precision=pkg.PREC_DF, **kw) as pdf:
        for c in (c32, p64, pdf):
            c.set_w(wa, wb)
            c.iterate(1)
        c32.set_w(wa, wb)
        t0 = time.perf_counter()
        # FP32 propagation floors the residual near 2e-5 (64^3); switch to
        # the polish at 3e-5 (measured: 48 FP64 polish iterations, against 76
        # from 1e-4), or as soon as FP32 stops making progress (at 128^3 the
        # floor sits at about 3e-5 and reaching it took 591 iterations)
        it32 = converge_until_floor(c32, 3e-5, max_it, budget_s)
        t32 = time.perf_counter() - t0
        w32 = (c32.wa, c32.wb)
        for name, pol, key in ((nm, {"fp64": p64, "df": pdf}[k], k) for nm, k in polishes):
            t1 = time.perf_counter()
            pol.copy_fields_from(c32)
            itp, fep, okp = converge_timed(pol, tol, max_it, budget_s)
            tp = time.perf_counter() - t1
            res = {"seconds": t32 + tp, "seconds_fp32": t32, "iterations_fp32": it32,
                   "iterations_polish": itp, "F": fep[0, 0],
                   "residual": float(pol.residual()[0][0]), "converged": okp,
                   "speedup": t64 / (t32 + tp)}
            res.update(compare_to_fp64(ref, state(pol, fep)))
            t1 = time.perf_counter()
            it7, fe, ok = converge_timed(pol, 1e-7, 1000, 40.0)
            tp7 = t32 + tp + time.perf_counter() - t1
            if ok and ref_t is not None:
                res["at_tol_1e-7"] = compare_to_fp64(ref_t, state(pol, fe))
                res["at_tol_1e-7"].update(seconds=tp7, iterations_polish=itp + it7,
                                          speedup=t64_7 / tp7)
            out[name] = res
        # errors of the FP32-propagation path against the FP64 path (the CPU
        # oracle's discretisation, matched to 1e-11) at the same fields: the
        # FP32 solve's end point
        ev = {}
        for c in (c32, p64):
            c.set_w(*w32)
            c.get_conc()
            ev[c] = (c.pha, c.phb, c.Q(), c.free_energy()[0])
        a, b = ev[c32], ev[p64]
        out["fp32_errors_vs_fp64_same_fields"] = {
            "phiA_rel": float(np.abs(a[0] - b[0]).max() / np.abs(b[0]).max()),
            "phiB_rel": float(np.abs(a[1] - b[1]).max() / np.abs(b[1]).max()),
            "Q_rel": float(abs(a[2][0] / b[2][0] - 1)),
            "F_abs": float(abs(a[3][0] - b[3][0])), "F_rel": float(abs(a[3][0] / b[3][0] - 1))}
    # the headline: the faster polish that meets the F criterion (1e-7)
    ok = [nm for nm, _ in polishes if out[nm]["converged"] and out[nm]["F_abs_diff"] < 1e-7]
    best = min(ok, key=lambda k: out[k]["seconds"]) if ok else polishes[0][0]
    out.update(method=best, speedup=out[best]["speedup"], F_abs_diff=out[best]["F_abs_diff"],
               phiA_rel_diff=out[best]["phiA_rel_diff"],
               phiA_rel_diff_shift_aligned=out[best]["phiA_rel_diff_shift_aligned"],
               Q_rel_diff=out[best]["Q_rel_diff"])
    t7 = out[best].get("at_tol_1e-7")
    if t7:
        out["at_tol_1e-7"] = {"speedup": t7["speedup"], "phiA_rel_diff": t7["phiA_rel_diff"],
                              "F_abs_diff": t7["F_abs_diff"]}
    out["clocks"] = clocks.stop()
    return out


def stress_leg(pkg, dev, relax=False, budget_s=60.0):
    """Config 3: hexagonal cylinders, f=0.3, chiN=25, 128x128x64, box
    Lx=4.2, Ly=Lx*sqrt(3), Lz=2.0, Ns=200, FP32 propagation with FP64
    reductions, Anderson m=20.  Converges the fields (FP32 floor 3e-5), then
    times the box stress (-d ln Q/dL from the stored propagators) and the
    checkpointed adjoint; checks the stress against an FP64 context and
    against central differences of FP64 ln Q with h = 1e-4 L.  With relax,
    also runs the stress-driven unit-cell relaxation of Lx, Ly."""
    import math
    from scft_gb300 import fields as fl
    nx, ny, nz, lx, lz = 128, 128, 64, 4.2, 2.0
    ly = lx * math.sqrt(3)
    kw = dict(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=25.0, fA=0.3, ds0=0.005,
              mixing=pkg.MIX_ANDERSON, anderson_history=20, device=dev)
    wa, wb = fl.hexagonal(nx, ny, nz, lx, ly, lz, 25.0, seed=0)
    out = {"config": "128x128x64 hexagonal cylinders, f=0.3, chiN=25, box 4.2 x 7.2746 x 2.0, "
                     "Ns=200, FP32 propagation, Anderson m=20"}
    with pkg.Context(precision=pkg.PREC_FP32, **kw) as c:
        c.set_w(wa, wb)
        t0 = time.perf_counter()
        it, fe, ok = converge_timed(c, 3e-5, 3000, budget_s)
        out["converge"] = {"seconds": time.perf_counter() - t0, "iterations": it,
                           "residual": float(c.residual()[0][0]), "F": fe[0, 0]}
        wa1, wb1 = c.wa, c.wb
        c.get_conc()
        c.stress()                                   # allocation, warm-up
        c.synchronize()
        t0 = time.perf_counter()
        s32 = c.stress()
        out["stress_fp32"] = {"dF_dL": s32[0].tolist(), "ms": (time.perf_counter() - t0) * 1e3}
        c.adjoint(None, None, 1.0)                   # allocation, warm-up
        for want_L in (True, False):
            t0 = time.perf_counter()
            c.adjoint(None, None, 1.0, want_L=want_L)
            out["adjoint_ms" + ("_with_box" if want_L else "_fields_only")] = \
                (time.perf_counter() - t0) * 1e3
        n_sl, by = c.adjoint_checkpoints(0)
        out["adjoint_memory"] = {"slices": n_sl, "bytes": by,
                                 "stored_propagators_bytes": 4 * (c.NsA + c.dNsB + 2) * nx * ny
                                 * nz * 4}
        out["sweep_ms_per_scf_iteration"] = c.time_iterations(3) / 3
    with pkg.Context(precision=pkg.PREC_FP64, **kw) as c:
        c.set_w(wa1, wb1)
        c.get_conc()
        s64 = c.stress()
        fd = []
        for a in range(3):
            L = [lx, ly, lz]
            h = 1e-4 * L[a]
            lnq = []
            for sg in (1, -1):
                Lp = list(L)
                Lp[a] += sg * h
                c.set_box(*Lp)
                c.set_w(wa1, wb1)
                c.get_conc()
                lnq.append(math.log(c.Q()[0]))
            fd.append(-(lnq[0] - lnq[1]) / (2 * h))
        den = max(abs(v) for v in fd)
        out["stress_fp64"] = s64[0].tolist()
        out["stress_fd_fp64_h1e-4L"] = fd
        out["rel_err_fp64_vs_fd"] = max(abs(a - b) for a, b in zip(s64[0], fd)) / den
        out["rel_err_fp32_vs_fp64"] = max(abs(a - b) for a, b in zip(s32[0], s64[0])) / den
        # the same stress at FP64 level in double-float arithmetic, and the
        # getConc + stress time of each precision at these fields
        c.set_box(lx, ly, lz)
        c.set_w(wa1, wb1)
        c.synchronize()
        t0 = time.perf_counter()
        c.get_conc()
        c.stress()
        t_prec = {"fp64": (time.perf_counter() - t0) * 1e3}
    with pkg.Context(precision=pkg.PREC_DF, **kw) as c:
        c.set_w(wa1, wb1)
        c.get_conc()
        c.stress()                       # warm-up (tables, buffers)
        c.set_w(wa1, wb1)
        c.synchronize()
        t0 = time.perf_counter()
        c.get_conc()
        sdf = c.stress()
        t_prec["df"] = (time.perf_counter() - t0) * 1e3
        out["stress_df"] = sdf[0].tolist()
        out["rel_err_df_vs_fp64"] = max(abs(a - b) for a, b in zip(sdf[0], s64[0])) / den
        out["getconc_plus_stress_ms"] = t_prec
    if relax:
        with pkg.Context(precision=pkg.PREC_FP32, **kw) as c:
            c.set_w(wa1, wb1)
            t0 = time.perf_counter()
            rounds, sig, fe = c.relax_cell(axes_mask=3, tol_w=3e-5, tol_stress=1e-5,
                                           max_outer=40, max_inner=2000)
            out["relax"] = {"seconds": time.perf_counter() - t0, "rounds": rounds,
                            "dF_dL": sig.tolist(), "F": fe[0], "box": c.box().tolist()}
    return out


def large_leg(pkg, dev, converge=False, budget_s=120.0):
    """Config 5: one 256^3 solve, lamellar/gyroid mixture init, f=0.45,
    chiN=22, box 8.0 Rg, Ns=400, FP32 propagation with FP64 Q and Anderson
    (history 30).  Throughput of 3 SCF iterations (device events) with the
    march phase's roofline; with converge, the time to the FP32 floor."""
    from scft_gb300 import fields as fl
    n, Lb = 256, 8.0
    # two unit cells per 8 Rg box: about the lamellar period at chiN = 22
    wa, wb = fl.mixture(n, n, n, Lb, Lb, Lb, 22.0, seed=0, periods=2)
    peak, peak_kind = load_peaks()
    with pkg.Context(nx=n, ny=n, nz=n, lx=Lb, ly=Lb, lz=Lb, hAB=22.0, fA=0.45, ds0=1.0 / 400,
                     precision=pkg.PREC_FP32, mixing=pkg.MIX_ANDERSON, anderson_history=30,
                     device=dev) as c:
        c.set_w(wa, wb)
        c.iterate(2)
        c.synchronize()
        c.profile_enable(16)
        ms = c.time_iterations(3) / 3
        march_ms, n_m, march_pts = c.profile_read()
        c.profile_enable(0)
        pts = 2 * (c.NsA + c.dNsB) * n ** 3
        sched, _ = c.schedule()
        out = {"config": "256^3 lamellar/gyroid mixture (two cells per box), f=0.45, chiN=22, "
                         "box 8.0 Rg, Ns=400 (NsA=180, dNsB=220), FP32 propagation, Anderson m=30",
               "ms_per_scf_iteration": ms, "gpt_step_per_s": pts / (ms / 1e3) / 1e9,
               "march_roofline_frac": march_pts / (march_ms / 1e3) * 12.0 / 1e9 / peak,
               "peak_kind": peak_kind, "schedule_flags": sched,
               "propagator_bytes": 4 * (2 * c.NsA + 2 * c.dNsB + 4) * n ** 3}
        if converge:
            c.set_w(wa, wb)
            t0 = time.perf_counter()
            it, fe, ok = converge_timed(c, 5e-5, 5000, budget_s)
            out["converge_to_5e-5"] = {"seconds": time.perf_counter() - t0, "iterations": it,
                                       "converged": ok, "residual": float(c.residual()[0][0]),
                                       "F": fe[0, 0]}
    return out


def precision_matched_leg(pkg, dev, iters=3):
    """The FP64-level paths on the benchmark workload (128^3 gyroid, Ns=200,
    simple mixing): plain FP64 and double-float (FP32-pair) propagation, in
    Gpt*step/s from device events around whole SCF iterations, for comparison
    with the reference's FP64 CUDA build at the same arithmetic accuracy."""
    from scft_gb300 import fields as fl
    wa, wb = fl.gyroid(N, N, N, L, L, L, CHIN, seed=0)
    out = {"what": "128^3 gyroid Ns=200, 1 SCF iteration per step, %d steps after a warm-up"
                   % iters}
    for name, prec in (("fp64", pkg.PREC_FP64), ("df", pkg.PREC_DF)):
        with pkg.Context(nx=N, ny=N, nz=N, lx=L, ly=L, lz=L, hAB=CHIN, fA=FA, ds0=DS,
                         precision=prec, device=dev) as c:
            c.set_w(wa, wb)
            c.iterate(2)
            c.synchronize()
            ms = c.time_iterations(iters) / iters
            pts = 2 * (c.NsA + c.dNsB) * N ** 3
            out[name] = {"ms_per_iteration": ms, "gpt_step_per_s": pts / (ms / 1e3) / 1e9}
    return out


def cufft_leg(dev, n=N, steps=50):
    """cuFFT comparison (timed only as a comparison, not used by the library):
    the same FP32 split step q <- W*irfftn(G*rfftn(W*q)) with torch.fft
    (cuFFT R2C/C2R) at n^3, one propagator, CUDA events on torch's stream."""
    import torch
    d = torch.device(f"cuda:{dev}")
    g = torch.Generator(device=d).manual_seed(0)
    W = 1.0 + 0.01 * torch.rand((n, n, n), device=d, generator=g)
    k = torch.fft.fftfreq(n, d=1.0 / n, device=d) * (2 * np.pi / L)
    kr = torch.fft.rfftfreq(n, d=1.0 / n, device=d) * (2 * np.pi / L)
    G = torch.exp(-DS * (k[:, None, None] ** 2 + k[None, :, None] ** 2 + kr[None, None, :] ** 2))
    q = torch.ones((n, n, n), device=d)
    for _ in range(5):
        q = W * torch.fft.irfftn(G * torch.fft.rfftn(W * q), s=(n, n, n))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(d)
    e0.record()
    for _ in range(steps):
        q = W * torch.fft.irfftn(G * torch.fft.rfftn(W * q), s=(n, n, n))
    e1.record()
    torch.cuda.synchronize(d)
    ms = e0.elapsed_time(e1) / steps
    return {"what": "torch.fft (cuFFT) FP32 split step, one propagator, %d^3" % n,
            "us_per_step": ms * 1e3, "gpt_step_per_s": n ** 3 / (ms / 1e3) / 1e9}


def batch_sweep_leg(pkg, dev, n_inst=64, iters=3, seed=4):
    """Config-4 phase-diagram sweep: 64 independent instances, grids drawn from
    {32^3, 48^3, 64^3}, chiN~U[12,30], f~U[0.25,0.5], box~U[3,5] Rg,
    Ns~U{100..200}, seeded random fields, FP32 propagation.  Aggregate
    Gpt*step/s of one group (one graph launch per iteration) against the same
    instances iterated one after another."""
    from scft_gb300 import fields as fl
    rng = np.random.default_rng(seed)
    ctxs, pts = [], 0
    for i in range(n_inst):
        n = int(rng.choice([32, 48, 64]))
        chin = float(rng.uniform(12, 30))
        f = float(rng.uniform(0.25, 0.5))
        box = float(rng.uniform(3.0, 5.0))
        ns = int(rng.integers(100, 201))
        # each member's march schedule is autotuned on its own grid
        c = pkg.Context(nx=n, ny=n, nz=n, lx=box, ly=box, lz=box, hAB=chin, fA=f, ds0=1.0 / ns,
                        precision=pkg.PREC_FP32, device=dev, flags=pkg.FLAG_AUTOTUNE)
        wa, wb = fl.random_fields(n, n, n, seed=1000 + i, scale=0.1 * chin)
        c.set_w(wa, wb)
        c.iterate(1)                      # capture the member's own march graph
        pts += 2 * (c.NsA + c.dNsB) * n ** 3
        ctxs.append(c)
    seq_ms = 0.0
    for c in ctxs:
        c.synchronize()
        seq_ms += c.time_iterations(iters)
    with pkg.Group(ctxs) as g:
        g.iterate(1)
        grp_ms = g.time_iterations(iters)
        launches = g.launch_count()
    for c in ctxs:
        c.close()
    seq = pts * iters / (seq_ms / 1e3) / 1e9
    grp = pts * iters / (grp_ms / 1e3) / 1e9
    return {"config": "%d instances, grids {32,48,64}^3, chiN U[12,30], f U[0.25,0.5], box "
                      "U[3,5], Ns U{100..200}, FP32, autotuned schedules, seed %d"
                      % (n_inst, seed),
            "sequential_gpt_step_per_s": seq, "group_gpt_step_per_s": grp,
            "speedup": grp / seq, "iterations": iters, "group_graph_launches": launches}


def run_ours(args):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    from scft_gb300 import fields as fl
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local if ws > 1 else 0
    prec = {"fp64": pkg.PREC_FP64, "df": pkg.PREC_DF}.get(args.precision, pkg.PREC_FP32)
    n, ds = args.grid, 1.0 / args.ns
    headline = (n == N and args.ns == 200 and args.mixing == "simple")
    mix = ({"mixing": pkg.MIX_ANDERSON, "anderson_history": 20, "anderson_start": 1e9}
           if args.mixing == "anderson" else {})
    ctx = pkg.Context(nx=n, ny=n, nz=n, lx=L, ly=L, lz=L, hAB=CHIN, fA=FA, ds0=ds,
                      precision=prec, device=dev, **mix)
    wa, wb = fl.gyroid(n, n, n, L, L, L, CHIN, seed=rank)
    ctx.set_w(wa, wb)
    pt_steps = 2 * (ctx.NsA + ctx.dNsB) * n ** 3

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if dist is not None:
            dist.barrier()

    # The clock sampler starts before the warm-up: nvidia-smi's start-up then
    # falls outside the timed region, and the GPU is busy from the first sample.
    clocks = ClockSampler(dev) if rank == 0 else None
    # warm-up (at least ~0.3 s so that the sampler is running)
    t_w = time.perf_counter()
    nw = 0
    while nw < args.warmup or time.perf_counter() - t_w < 0.3:
        ctx.iterate(1)
        nw += 1
        if nw % 4 == 0:
            ctx.synchronize()
    barrier()

    # ---- timed region: K steps, device events on the library's stream
    l0 = ctx.launch_count()
    ctx.profile_enable(4 * args.steps + 8)
    t0 = time.perf_counter()
    ms = ctx.time_iterations(args.steps)
    wall = time.perf_counter() - t0
    march_ms, n_marches, march_pts = ctx.profile_read()
    ctx.profile_enable(0)
    launches = ctx.launch_count() - l0
    barrier()
    clk = clocks.stop() if clocks else None
    t_max = max_over_ranks(ms, dist, f"cuda:{dev}")
    value = ws * pt_steps * args.steps / (t_max / 1e3) / 1e9

    # ---- end-to-end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hw_a = torch.from_numpy(wa.reshape(-1)).pin_memory()
        hw_b = torch.from_numpy(wb.reshape(-1)).pin_memory()
        ho_a = torch.empty(n ** 3, dtype=torch.float64).pin_memory()
        ho_b = torch.empty(n ** 3, dtype=torch.float64).pin_memory()
        import ctypes as C
        dptr = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_double))
        out5 = np.empty(5)
        e2e_steps = max(1, min(args.steps, 10))

        def e2e_step():
            ctx._ck(ctx.lib.scft_set_field(ctx.h, pkg.FIELD_WA, dptr(hw_a)))
            ctx._ck(ctx.lib.scft_set_field(ctx.h, pkg.FIELD_WB, dptr(hw_b)))
            ctx._ck(ctx.lib.scft_iterate(ctx.h, 1, out5.ctypes.data_as(C.POINTER(C.c_double))))
            ctx._ck(ctx.lib.scft_get_field(ctx.h, pkg.FIELD_PHA, dptr(ho_a)))
            ctx._ck(ctx.lib.scft_get_field(ctx.h, pkg.FIELD_PHB, dptr(ho_b)))

        e2e_step()                      # warm-up: first touch of the pinned buffers
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        barrier()
        e2e_s = max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{dev}")
        e2e = {"value": ws * pt_steps * e2e_steps / e2e_s / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": 2 * 8 * n ** 3, "d2h_bytes_per_step": 2 * 8 * n ** 3 + 5 * 8,
               "steps": e2e_steps,
               "path": "scft_set_field x2 (pinned host) + scft_iterate(1) + scft_get_field x2"}

    if rank == 0:
        peak, peak_kind = load_peaks()
        bpp = BYTES_PER_PT_STEP[args.precision]
        march_rate = march_pts / (march_ms / 1e3)          # pt-steps/s inside marches
        achieved = march_rate * bpp / 1e9                  # GB/s, algorithmic bytes
        workload = WORKLOAD if headline else (
            f"{n}^3 gyroid (f=0.36, chiN=18, box 3.8), Ns={args.ns}, {args.mixing} mixing: a "
            f"case for profiling, not the headline")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "fp64": "f64"}.get(args.precision, "f32x2 (double-float)"),
            "data": "synthetic",
            "config": {"workload": workload, "grid": [n, n, n], "Ns": args.ns, "batch": 1,
                       "propagation": args.precision,
                       "reductions": "fp64 (Q, F, mixing); phi contour sum compensated",
                       "l2": "inputs larger than L2: each step (one SCF iteration) stores "
                             "and re-reads %.1f GB of propagator slices (2*(NsA+dNsB+2) slices "
                             "of the four marches) through HBM"
                             % (2 * (ctx.NsA + ctx.dNsB + 2) * n ** 3 *
                                (4 if args.precision == "fp32" else 8) / 1e9),
                       "parallelism": f"replicas x{ws} (no exchange step)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": TRAFFIC_PER_STEP if (headline and args.precision == "fp32")
                         else None,
                         "traffic_note": TRAFFIC_NOTE,
                         "peak_kind": peak_kind,
                         "kernel": "propagator march (sovDifFft): one fused launch per contour "
                                   "step at 128^3 (k_xyxy / k_zz alternating)",
                         "bytes_per_point_step": bpp,
                         "march_ms_avg": march_ms / max(n_marches, 1),
                         "marches_timed": n_marches},
            "cpu_baseline": cpu_baseline() if not args.no_cpu else None,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": dict(clk or {}, window="sampled every 50 ms from the start of the warm-up "
                                            "to the end of the timed region",
                           warmup_iterations_run=nw),
            "wall_s_timed": wall,
            "converge": (converge_leg(pkg, dev, pin=True) if (not args.no_converge and ws == 1)
                         else None),
            "converge_128": (converge_leg(pkg, dev, n=N, budget_s=120.0,
                                          polishes=(("fp32_df_polish", "df"),), pin=True)
                             if (headline and not args.no_converge and ws == 1) else None),
            "batch_sweep": (batch_sweep_leg(pkg, dev) if (not args.no_sweep and ws == 1)
                            else None),
            "stress_adjoint": (stress_leg(pkg, dev, relax=args.relax)
                               if (not args.no_stress and ws == 1) else None),
            "cufft_comparison": (cufft_leg(dev) if (headline and ws == 1 and not args.no_cufft)
                                 else None),
            "precision_matched": (precision_matched_leg(pkg, dev)
                                  if (headline and ws == 1 and not args.no_prec) else None),
            "large_256": (large_leg(pkg, dev, converge=args.large_converge)
                          if (headline and ws == 1 and not args.no_large) else None),
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "df"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--grid", type=int, default=N, help="grid edge (profiling cases only)")
    ap.add_argument("--ns", type=int, default=200, help="contour steps 1/ds (profiling only)")
    ap.add_argument("--mixing", default="simple", choices=["simple", "anderson"],
                    help="field update of the timed iterations (anderson: profiling only)")
    ap.add_argument("--no-sweep", action="store_true",
                    help="skip the 64-instance heterogeneous sweep leg")
    ap.add_argument("--no-converge", action="store_true",
                    help="skip the seconds-to-converge leg (FP64 vs FP32+FP64 polish)")
    ap.add_argument("--no-stress", action="store_true",
                    help="skip the config-3 stress / adjoint leg")
    ap.add_argument("--no-cufft", action="store_true", help="skip the cuFFT comparison leg")
    ap.add_argument("--no-large", action="store_true", help="skip the 256^3 Ns=400 leg")
    ap.add_argument("--no-prec", action="store_true",
                    help="skip the FP64 / double-float rates at 128^3")
    ap.add_argument("--no-ref-cuda", action="store_true",
                    help="reference arm: skip the reference's own CUDA build")
    ap.add_argument("--large-converge", action="store_true",
                    help="add the 256^3 convergence run to the large leg (minutes)")
    ap.add_argument("--relax", action="store_true",
                    help="add the unit-cell relaxation to the stress leg (minutes)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
