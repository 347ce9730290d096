"""CPU oracle for the diblock-copolymer SCFT hot path.

TEST INFRASTRUCTURE ONLY.  This module is a float64 NumPy restatement of the
reference's algorithm (ren5885a/SCFT_Ver1.01).  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may
import it, and only as the checker / timed CPU baseline.  The product path
(the CUDA library behind ``include/scft_capi.h``) never calls it.

Parity pinning: the reference ships no tests, golden vectors or fixtures for
this path.  The oracle is pinned (a) by known-answer tests derived from the
mathematics (see ``tests/test_oracle.py``) and (b) against outputs of the
reference's own CUDA kernels + cuFFT, compiled from the reference sources by
``oracle/Makefile`` and driven by ``oracle/ref_harness.cpp`` on a GB300; those
outputs are committed as ``tests/golden/ref_*.npz`` by
``tests/golden/make_ref_golden.py``.

Every function cites the reference file:line it restates.  Layout: fields are
``[batch][Nz][Ny][Nx]`` (x fastest), exactly the reference's ``ijk=(k*Ny+j)*Nx+i``
order (init_cuda.cu:422).  Propagators are returned contour-outer
``[batch][ns+1][Nz][Ny][Nx]`` (the reference stores them s-fastest,
``g[b][r][s]``, cuda_aid.cu:237; only the memory order differs).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# struct.h:11 -- the reference's (truncated) value of pi; kept for parity.
PI_REF = 3.1415926535


@dataclass
class Params:
    """The ``ab.txt`` keys (init.cpp:86-92) plus the hard-coded constants.

    ``wopt``/``wcmp`` are the simple-mixing constants hard-coded in
    ``phi_w`` (cuda_aid.cu:395-396); ``aver_it`` is ``AverIt`` (init.cpp:39).
    """

    nx: int = 32
    ny: int = 32
    nz: int = 32
    lx: float = 4.0
    ly: float = 4.0
    lz: float = 4.0
    hAB: float = 20.0          # xN
    fA: float = 0.5            # fa
    ds0: float = 0.01
    batch: int = 1             # Num_SCFT
    intag: int = 1024
    wopt: float = 0.05
    wcmp: float = 0.10
    aver_it: int = 10
    simpson: bool = False      # contour sums with Simpson weights (no reference counterpart)

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def M(self):
        return self.nx * self.ny * self.nz

    @property
    def NsA(self):
        # init_cuda.cu:330
        return int(self.fA / self.ds0 + 1.0e-8)

    @property
    def dNsB(self):
        # init_cuda.cu:329,331 (dfB = 1 - fA)
        return int((1.0 - self.fA) / self.ds0 + 1.0e-8)

    @property
    def ds2(self):
        # init_cuda.cu:328
        return self.ds0 / 2


# ---------------------------------------------------------------- config I/O

def parse_ab_txt(text: str) -> Params:
    """Parse the ``ab.txt`` format read at init.cpp:86-92."""
    p = Params()
    vals = {}
    for line in text.splitlines():
        for part in line.split(","):
            if "=" in part:
                k, v = part.split("=", 1)
                vals[k.strip()] = v.strip()
    p.intag = int(vals["intag"])
    p.hAB = float(vals["xN"])
    p.fA = float(vals["fa"])
    p.lx, p.ly, p.lz = float(vals["lx"]), float(vals["ly"]), float(vals["lz"])
    p.nx, p.ny, p.nz = int(vals["Nx"]), int(vals["Ny"]), int(vals["Nz"])
    p.ds0 = float(vals["ds0"])
    p.batch = int(vals["batch"])
    return p


def format_g(x: float) -> str:
    """C printf ``%g`` (6 significant digits)."""
    return "%g" % x


def write_pha_dat(path, p: Params, pha, phb, wa, wb):
    """Writer of ``pha_%d.dat`` (cuda_scft.cu:233-243)."""
    dx, dy, dz = p.lx / p.nx, p.ly / p.ny, p.lz / p.nz
    with open(path, "w") as f:
        f.write("Nx=%d, Ny=%d, Nz=%d\n" % (p.nx, p.ny, p.nz))
        f.write("dx=%g, dy=%g, dz=%g\n" % (dx, dy, dz))
        for a, b, c, d in zip(pha.ravel(), phb.ravel(), wa.ravel(), wb.ravel()):
            f.write("%g %g %g %g\n" % (a, b, c, d))


def read_phi_dat(path, M):
    """Reader of ``phi_%d.dat`` (init_cuda.cu:435-456): 2 header lines, then
    M lines ``pha phb wa wb``."""
    with open(path) as f:
        f.readline()
        f.readline()
        data = np.loadtxt(f, max_rows=M)
    data = data.reshape(M, 4)
    return data[:, 0].copy(), data[:, 1].copy(), data[:, 2].copy(), data[:, 3].copy()


# ----------------------------------------------------------- spectral tables

def k2_axis(n: int, length: float) -> np.ndarray:
    """Squared wave numbers of one axis (init_cuda.cu:398-418).

    Bins ``i <= n/2-1`` get ``+i``, bins ``i >= n/2`` get ``i-n`` (so a
    length-1 axis gets ``-1``: the reference's Nz=1 behaviour).
    """
    d = length / n
    k = np.empty(n)
    for i in range(0, n // 2):
        k[i] = 2 * PI_REF * i * 1.0 / n / d
    for i in range(n // 2, n):
        k[i] = 2 * PI_REF * (i - n) * 1.0 / d / n
    return k * k


def kxyzdz(p: Params) -> np.ndarray:
    """``kxyzdz[k][j][i] = exp(-ds0*(kx2[i]+ky2[j]+kz2[k]))`` (init_cuda.cu:420-428)."""
    kx = k2_axis(p.nx, p.lx)
    ky = k2_axis(p.ny, p.ly)
    kz = k2_axis(p.nz, p.lz)
    ksq = (kx[None, None, :] + ky[None, :, None]) + kz[:, None, None]
    return np.exp(-p.ds0 * ksq)


def kxyzdz_half(p: Params) -> np.ndarray:
    """The table as ``sufaceField_go`` indexes it for the D2Z half spectrum:
    ``ijkr = ix + iy*Nx + iz*Nx*Ny`` with ``ix < Nx/2+1`` (cuda_aid.cu:312-325)."""
    return kxyzdz(p)[:, :, : p.nx // 2 + 1]


# ------------------------------------------------------------ hot-path steps

def average_value(w: np.ndarray) -> np.ndarray:
    """``average_value`` (cuda_scft.cu:14-59): per instance, ``w -= sum(w)/M``
    (reduce3, cuda_aid.cuh:36-80, then minus_average, cuda_aid.cu:365-380)."""
    b = w.shape[0]
    flat = w.reshape(b, -1)
    s = flat.sum(axis=1)
    return (flat - (s / flat.shape[1])[:, None]).reshape(w.shape)


def sov_dif_fft(q_init: np.ndarray, w: np.ndarray, ns: int, sign: int, p: Params,
                kdz_half: np.ndarray | None = None) -> np.ndarray:
    """One propagator march (``sovDifFft``, cuda_scft.cu:435-563).

    ``q_init``/``w``: ``[batch][Nz][Ny][Nx]``.  Returns ``[batch][ns+1][...]``.
    sign=+1: q[0]=q_init, for iz=1..ns: q[iz] from q[iz-1] (cuda_scft.cu:458-494).
    sign=-1: q[ns]=q_init, for iz=ns-1..0: q[iz] from q[iz+1] (:506-545).
    Each step: in = q*wdz (initilize_in_go, cuda_aid.cu:227-241); D2Z;
    out *= kxyzdz (sufaceField_go, :306-328); Z2D; q = in*wdz/M
    (in_to_g_go, :346-361).  numpy's irfftn includes the 1/M.
    """
    if kdz_half is None:
        kdz_half = kxyzdz_half(p)
    wdz = np.exp(-w * p.ds2)                    # initilize_wdz, cuda_aid.cu:242-257
    b = w.shape[0]
    q = np.empty((b, ns + 1) + p.shape)
    axes = (1, 2, 3)
    if sign == 1:
        q[:, 0] = q_init                        # initilize_q, cuda_aid.cu:259-272
        order = [(iz, iz - 1) for iz in range(1, ns + 1)]
    elif sign == -1:
        q[:, ns] = q_init                       # initilize_q_inverse, cuda_aid.cu:274-287
        order = [(iz, iz + 1) for iz in range(ns - 1, -1, -1)]
    else:
        raise ValueError("sign must be +1 or -1")
    for dst, src in order:
        spec = np.fft.rfftn(q[:, src] * wdz, axes=axes)
        spec *= kdz_half[None]
        q[:, dst] = np.fft.irfftn(spec, s=p.shape, axes=axes) * wdz
    return q


@dataclass
class Conc:
    pha: np.ndarray
    phb: np.ndarray
    Q: np.ndarray            # per instance, ql/M (cuda_scft.cu:124)
    qa: np.ndarray
    qcb: np.ndarray
    qb: np.ndarray
    qca: np.ndarray
    wa: np.ndarray           # wa after getConc's own average_value (cuda_scft.cu:71)


def contour_weights(n: int, simpson: bool = False) -> np.ndarray:
    """Weights of the contour points s = 0..n of a block of n steps.

    Trapezoid (``w_to_phi_go``, cuda_aid.cu:87-107): 1/2 at both ends, 1
    inside; the n == 0 block has the single weight 1/2 (cuda_aid.cu:91).
    Simpson (an option without a reference counterpart): the composite 1/3
    rule for even n; for odd n >= 3 the 1/3 rule over the first n-3 steps and
    the 3/8 rule over the last three; n == 1 stays trapezoid.  The weights of
    a block with n >= 1 sum to n."""
    if n == 0:
        return np.array([0.5])
    if not simpson or n == 1:
        w = np.ones(n + 1)
        w[0] = w[-1] = 0.5
        return w
    m = n if n % 2 == 0 else n - 3
    w = np.zeros(n + 1)
    if m > 0:
        w[1:m:2] = 4.0 / 3.0
        w[2:m:2] = 2.0 / 3.0
        w[0] += 1.0 / 3.0
        w[m] += 1.0 / 3.0
    if m < n:
        w[m] += 3.0 / 8.0
        w[m + 1] += 9.0 / 8.0
        w[m + 2] += 9.0 / 8.0
        w[n] += 3.0 / 8.0
    return w


def contour_sum(q: np.ndarray, qc: np.ndarray, simpson: bool = False) -> np.ndarray:
    """sum_s w_s q(s) qc(s) over a block, ``q``/``qc``: ``[batch][ns+1][...]``."""
    w = contour_weights(q.shape[1] - 1, simpson)
    return np.tensordot(w, np.moveaxis(q * qc, 1, 0), axes=1)


def trapezoid_sum(q: np.ndarray, qc: np.ndarray) -> np.ndarray:
    """Contour sum of ``w_to_phi_go`` (cuda_aid.cu:87-107): weights 1/2 at both
    ends, 1 inside.  ``q``/``qc``: ``[batch][ns+1][...]``."""
    prod = q * qc
    if prod.shape[1] == 1:          # ns == 0: iz==0 is also iz==ns (cuda_aid.cu:91)
        return 0.5 * prod[:, 0]
    s = 0.5 * prod[:, 0] + 0.5 * prod[:, -1]
    if prod.shape[1] > 2:
        s = s + prod[:, 1:-1].sum(axis=1)
    return s


def get_conc(wa: np.ndarray, wb: np.ndarray, p: Params, kdz_half=None) -> Conc:
    """``getConc`` (cuda_scft.cu:61-138)."""
    if kdz_half is None:
        kdz_half = kxyzdz_half(p)
    wa = average_value(wa)                                    # :71
    ones = np.ones_like(wa)                                   # qInt_init, :77
    qa = sov_dif_fft(ones, wa, p.NsA, +1, p, kdz_half)        # :83
    qcb = sov_dif_fft(ones, wb, p.dNsB, -1, p, kdz_half)      # :86
    qb = sov_dif_fft(qa[:, p.NsA], wb, p.dNsB, +1, p, kdz_half)   # qa_to_qInt :93, :99
    qca = sov_dif_fft(qcb[:, 0], wa, p.NsA, -1, p, kdz_half)      # qa_to_qInt2 :106, :112
    b = wa.shape[0]
    ql = qb[:, p.dNsB].reshape(b, -1).sum(axis=1)             # cal_ql, :118
    Q = ql / p.M                                              # :124
    ffl = p.ds0 / Q                                           # :125
    if p.simpson:
        pha = ffl[:, None, None, None] * contour_sum(qa, qca, True)
        phb = ffl[:, None, None, None] * contour_sum(qb, qcb, True)
    else:
        pha = ffl[:, None, None, None] * trapezoid_sum(qa, qca)   # w_to_phi_go, :130
        phb = ffl[:, None, None, None] * trapezoid_sum(qb, qcb)
    return Conc(pha, phb, Q, qa, qcb, qb, qca, wa)


def phi_w(wa, wb, pha, phb, hAB, wopt=0.05, wcmp=0.10):
    """Simple mixing (``phi_w``, cuda_aid.cu:382-416).  Returns the updated
    fields and the residuals (waDiff, wbDiff) before scaling by wopt."""
    eta = (wa + wb - hAB) / 2
    psum = 1.0 - pha - phb
    wad = hAB * phb + eta - wa
    wbd = hAB * pha + eta - wb
    wad = wad - wcmp * psum
    wbd = wbd - wcmp * psum
    return wa + wopt * wad, wb + wopt * wbd, wad, wbd


def phi_w_constrained(wa, wb, pha, phb, target, hAB, lam):
    """``phi_w_constrained`` (cuda_aid.cu:418-452): phi_w plus a penalty
    lam*(phiA - target) on wA and lam*(phiB - (1 - target)) on wB, with the
    kernel's own wopt 0.05 and wcmp 0.10."""
    wopt, wcmp = 0.050, 0.10
    eta = (wa + wb - hAB) / 2
    psum = 1.0 - pha - phb
    wad = hAB * phb + eta - wa + lam * (pha - target)
    wbd = hAB * pha + eta - wb + lam * (phb - (1 - target))
    wad = wad - wcmp * psum
    wbd = wbd - wcmp * psum
    return wa + wopt * wad, wb + wopt * wbd


def phi_w_constrained_ex(wa, wb, pha, phb, target, hAB):
    """``phi_w_constrainedEx`` (cuda_aid.cu:454-490): the exchange-field form
    with wum = -hAB(2 target - 1) - (wA - wB) and the kernel's own wopt 1.60,
    wcmp 0.50."""
    wopt, wcmp = 1.60, 0.50
    wum = -hAB * (target * 2 - 1) - (wa - wb)
    eta = (wa + wb - hAB + wum) / 2
    psum = 1.0 - pha - phb
    psum1 = pha - target
    wad = hAB * (1 - target) + eta - wa - wum
    wbd = hAB * target + eta - wb
    wad = wad - (2.0 * wcmp * psum - 2.0 * wcmp * psum1)
    wbd = wbd - 2 * wcmp * psum1
    return wa + wopt * wad, wb + wopt * wbd


def vtk_text(source, nx, ny, nz, dx, dy, dz, diff):
    """Text of the converter's output (vtk.c:54-76): header, then phiA - phiB
    as ``%7.4lf `` per point with x fastest and one line per (z, y) row."""
    out = ["# vtk DataFile Version 3.0\n",
           "# comment: converted from file %s\n" % source,
           "ASCII\n", "DATASET STRUCTURED_POINTS\n",
           "DIMENSIONS %d %d %d\n" % (nx, ny, nz),
           "ORIGIN 0.000000 0.000000 0.000000\n",
           "SPACING %.6f %.6f %.6f\n\n" % (dx, dy, dz),
           "POINT_DATA %d\n" % (nx * ny * nz),
           "SCALARS scalars float\n", "LOOKUP_TABLE default\n\n"]
    d = np.asarray(diff, dtype=np.float64).reshape(nz * ny, nx)
    for row in d:
        out.append("".join("%7.4f " % v for v in row) + "\n")
    return "".join(out)


def convert_pha_to_vtk(pha_path, source=None):
    """The converter (vtk.c:4-81) on a pha file: returns the VTK text."""
    with open(pha_path) as f:
        h1 = f.readline()
        h2 = f.readline()
        nx, ny, nz = (int(t.split("=")[1]) for t in h1.strip().split(","))
        dx, dy, dz = (float(t.split("=")[1]) for t in h2.strip().split(","))
        data = np.loadtxt(f, max_rows=nx * ny * nz).reshape(-1, 4)
    return vtk_text(source or pha_path, nx, ny, nz, dx, dy, dz, data[:, 0] - data[:, 1])


def free_energy(wa, wb, pha, phb, Q, hAB):
    """The free-energy block of ``Free`` (cuda_scft.cu:190-221), per instance:
    returns (F, F_AB, F_W, F_S, inCompMax)."""
    b = wa.shape[0]
    pa, pb = pha.reshape(b, -1), phb.reshape(b, -1)
    a, bb = wa.reshape(b, -1), wb.reshape(b, -1)
    M = pa.shape[1]
    incomp = np.abs(1 - pa - pb).max(axis=1)
    fAB = (hAB * pa * pb).sum(axis=1) / M
    fW = -(a * pa + bb * pb).sum(axis=1) / M
    fS = -np.log(Q)
    return fAB + fW + fS, fAB, fW, fS, incomp


@dataclass
class FreeResult:
    wa: np.ndarray
    wb: np.ndarray
    pha: np.ndarray
    phb: np.ndarray
    Q: np.ndarray
    log: list = field(default_factory=list)   # (iter, b, F, FAB, FW, FS, incomp)


# ------------------------------------------------------------ derivatives
# No reference counterpart: the checks of the CUDA adjoint and stress.  The
# box enters only through kxyzdz (init_cuda.cu:394-428), k_a = 2 pi m / L_a.

def with_box(p: Params, lx=None, ly=None, lz=None) -> Params:
    import dataclasses
    return dataclasses.replace(p, lx=p.lx if lx is None else lx, ly=p.ly if ly is None else ly,
                               lz=p.lz if lz is None else lz)


def conc_functional(wa, wb, p: Params, pha_bar=None, phb_bar=None, Q_bar=None):
    """J = sum(pha_bar*phiA) + sum(phb_bar*phiB) + sum_b Q_bar[b]*Q[b] of
    getConc (cuda_scft.cu:61-138) at (wa, wb, box of p)."""
    c = get_conc(wa, wb, p)
    J = 0.0
    if pha_bar is not None:
        J += float((pha_bar * c.pha).sum())
    if phb_bar is not None:
        J += float((phb_bar * c.phb).sum())
    if Q_bar is not None:
        J += float((np.asarray(Q_bar) * c.Q).sum())
    return J


def stress_fd(wa, wb, p: Params, h_rel=1e-4):
    """Central finite differences of -ln Q per box axis, h = h_rel * L:
    -> [batch][3]."""
    out = np.zeros((wa.shape[0], 3))
    lens = (p.lx, p.ly, p.lz)
    for a in range(3):
        h = h_rel * lens[a]
        Qs = []
        for sgn in (+1, -1):
            L = list(lens)
            L[a] += sgn * h
            Qs.append(get_conc(wa, wb, with_box(p, *L)).Q)
        out[:, a] = -(np.log(Qs[0]) - np.log(Qs[1])) / (2 * h)
    return out


def stress_spectral(wa, wb, p: Params):
    """Analytic SCFT stress -d ln Q/dL_a at fixed fields: sum over contour
    steps of <q+(s), W (dK/dL_a) W q(s-1)> / (M Q), with dK/dL_a the
    diffusion filter whose Gaussian factor is multiplied by 2 ds k_a^2/L_a.
    -> [batch][3]."""
    c = get_conc(wa, wb, p)
    G = kxyzdz_half(p)
    k2 = [k2_axis(p.nx, p.lx)[None, None, : p.nx // 2 + 1],
          k2_axis(p.ny, p.ly)[None, :, None], k2_axis(p.nz, p.lz)[:, None, None]]
    lens = (p.lx, p.ly, p.lz)
    dG = [G * 2 * p.ds0 * k2[a] / lens[a] for a in range(3)]
    axes = (1, 2, 3)
    out = np.zeros((wa.shape[0], 3))
    blocks = ((c.qa, c.qca, c.wa, p.NsA), (c.qb, c.qcb, wb, p.dNsB))
    for q, qc, w, ns in blocks:
        W = np.exp(-w * p.ds2)
        for s in range(1, ns + 1):
            U = np.fft.rfftn(W * q[:, s - 1], axes=axes)
            for a in range(3):
                t = W * np.fft.irfftn(U * dG[a][None], s=p.shape, axes=axes)
                out[:, a] += (t * qc[:, s]).reshape(wa.shape[0], -1).sum(axis=1)
    return -out / (p.M * c.Q[:, None])


def free_energy_of(wa, wb, p: Params):
    """F of Free's formula (cuda_scft.cu:190-221) with phi and Q of getConc at
    these fields: -> [batch]."""
    c = get_conc(wa, wb, p)
    return free_energy(c.wa, wb, c.pha, c.phb, c.Q, p.hAB)[0]


def free_loop(wa, wb, p: Params, max_it: int, writer=None) -> FreeResult:
    """``Free`` (cuda_scft.cu:140-269): ``max_it`` SCF iterations of
    average_value(wa), average_value(wb), getConc, phi_w; every ``AverIt``
    iterations the free energy (computed with the *updated* w and the
    pre-update phi and Q, as the reference does) is logged; every
    ``10*AverIt`` iterations ``writer(iter, b, pha, phb, wa, wb)`` is called
    (the pha_%d.dat dump, :233-243)."""
    kdz = kxyzdz_half(p)
    res = FreeResult(wa, wb, None, None, None)
    pha = phb = Q = None
    for it in range(1, max_it + 1):
        wa = average_value(wa)                                 # :170
        wb = average_value(wb)                                 # :172
        c = get_conc(wa, wb, p, kdz)                           # :174
        wa, pha, phb, Q = c.wa, c.pha, c.phb, c.Q
        wa, wb, _, _ = phi_w(wa, wb, pha, phb, p.hAB, p.wopt, p.wcmp)   # :182
        if it % p.aver_it == 0:
            F, fAB, fW, fS, inc = free_energy(wa, wb, pha, phb, Q, p.hAB)
            for b in range(wa.shape[0]):
                res.log.append((it, b, F[b], fAB[b], fW[b], fS[b], inc[b]))
            if writer is not None and it % (p.aver_it * 10) == 0:
                for b in range(wa.shape[0]):
                    writer(it, b, pha[b], phb[b], wa[b], wb[b])
    res.wa, res.wb, res.pha, res.phb, res.Q = wa, wb, pha, phb, Q
    return res


def format_free_line(gpu_index, b, it, F, fAB, fW, fS, inc):
    """The progress line printed at cuda_scft.cu:221."""
    return "GPU %d batch %d: %5d : %.8e, %.8e, %.8e,%.8e, %.8e" % (
        gpu_index, b, it, F, fAB, fW, fS, inc)


# ---------------------------------------------------- CPU baseline (timed)

def iteration_cpu(wa, wb, p: Params, workers: int | None = None):
    """One full SCF iteration with scipy.fft (same arithmetic as free_loop's
    body, threaded FFTs).  Used only by bench.py's CPU-baseline legs."""
    import scipy.fft as sfft
    workers = workers or os.cpu_count()
    kdz = kxyzdz_half(p)[None]
    axes = (1, 2, 3)

    def march(q0, w, ns, sign):
        wdz = np.exp(-w * p.ds2)
        q = np.empty((w.shape[0], ns + 1) + p.shape)
        if sign == 1:
            q[:, 0] = q0
            order = [(i, i - 1) for i in range(1, ns + 1)]
        else:
            q[:, ns] = q0
            order = [(i, i + 1) for i in range(ns - 1, -1, -1)]
        for dst, src in order:
            spec = sfft.rfftn(q[:, src] * wdz, axes=axes, workers=workers)
            spec *= kdz
            q[:, dst] = sfft.irfftn(spec, s=p.shape, axes=axes, workers=workers) * wdz
        return q

    wa = average_value(average_value(wa))
    wb = average_value(wb)
    ones = np.ones_like(wa)
    qa = march(ones, wa, p.NsA, 1)
    qcb = march(ones, wb, p.dNsB, -1)
    qb = march(qa[:, p.NsA], wb, p.dNsB, 1)
    qca = march(qcb[:, 0], wa, p.NsA, -1)
    Q = qb[:, p.dNsB].reshape(wa.shape[0], -1).sum(axis=1) / p.M
    ffl = p.ds0 / Q
    pha = ffl[:, None, None, None] * trapezoid_sum(qa, qca)
    phb = ffl[:, None, None, None] * trapezoid_sum(qb, qcb)
    wa, wb, _, _ = phi_w(wa, wb, pha, phb, p.hAB, p.wopt, p.wcmp)
    return wa, wb, pha, phb, Q


def pt_steps_per_iteration(p: Params) -> int:
    """Grid points x contour steps of one SCF iteration: the four marches
    take NsA + dNsB + dNsB + NsA steps over batch*M points."""
    return 2 * (p.NsA + p.dNsB) * p.M * p.batch


def reduce3_quirk_sum(x: np.ndarray, threads: int) -> float:
    """The reference's ``reduce3`` block sum (cuda_aid.cuh:36-80) for a thread
    count that is not a power of two: the shared-memory tree halving drops
    elements, so the result differs from the true sum.  Used to document the
    quirk; the GPU path computes the true sum."""
    n = x.size
    chunk = n // threads + 1
    sdata = np.zeros(threads)
    for t in range(threads):
        lo = t * chunk
        hi = min(lo + chunk, n)
        if lo < n:
            sdata[t] = x[lo:hi].sum()
    s = threads // 2
    while s > 0:
        sdata[:s] = sdata[:s] + sdata[s:2 * s]
        s >>= 1
    return float(sdata[0])


def factor_decompose_1024(n: int) -> int:
    """Largest divisor of n that is <= 1024 (what factor_decompose_1024,
    init_cuda.cu:24-80, computes: the thread count of the reference's
    reductions and elementwise kernels)."""
    best = 1
    for d in range(1, min(n, 1024) + 1):
        if n % d == 0:
            best = d
    return best


# --------------------------------------------- convergence and Anderson mixing
# No reference counterpart (the reference runs a fixed MaxIT with phi_w,
# cuda_scft.cu:167-253).  Residual = phi_w's direction before the wopt step
# (cuda_aid.cu:398-408).  Anderson mixing: Anderson (1965) as used for SCFT by
# Thompson et al. (2004) and Matsen (2009), with an (m+1)-slot ring of (w, d).

def residual(wa, wb, pha, phb, hAB, wcmp=0.10):
    """(dA, dB, err_max[b], err_rms[b], cA, cB): dA, dB are phi_w's raw
    directions; cA, cB the same with their per-instance means removed.  The
    field mean is a gauge freedom that average_value removes every iteration
    (for f != 1/2 the raw direction carries the constant chiN*(1/2 - f)), so
    the norms and the Anderson history use the mean-free residual."""
    eta = (wa + wb - hAB) / 2
    psum = 1.0 - pha - phb
    da = hAB * phb + eta - wa
    db = hAB * pha + eta - wb
    da = da - wcmp * psum
    db = db - wcmp * psum
    b = wa.shape[0]
    ca = da - da.reshape(b, -1).mean(axis=1).reshape((b,) + (1,) * (da.ndim - 1))
    cb = db - db.reshape(b, -1).mean(axis=1).reshape((b,) + (1,) * (db.ndim - 1))
    mx = np.maximum(np.abs(ca).reshape(b, -1).max(axis=1), np.abs(cb).reshape(b, -1).max(axis=1))
    rms = np.sqrt(((ca * ca).reshape(b, -1).sum(axis=1) + (cb * cb).reshape(b, -1).sum(axis=1))
                  / (2.0 * da[0].size))
    return da, db, mx, rms, ca, cb


def anderson_weights(G, c, hist, m1, err_max, start, lam, wopt):
    """Per-instance slot weights a[m1] and step; simple step when err_max >=
    start or no history (mirrors the device solve, including its 1e-12
    diagonal shift)."""
    a = np.zeros(m1)
    if hist == 0 or not (err_max < start):
        a[c] = 1.0
        return a, wopt
    slot = lambda i: (c - i) % m1
    n = hist
    U = np.empty((n, n))
    V = np.empty(n)
    gcc = G[c, c]
    for i in range(n):
        si = slot(i + 1)
        V[i] = gcc - G[c, si]
        for j in range(n):
            sj = slot(j + 1)
            U[i, j] = gcc - G[c, si] - G[c, sj] + G[si, sj]
    dmax = np.abs(np.diag(U)).max()
    U = U + np.eye(n) * (1e-12 * dmax + 1e-300)
    x = np.linalg.solve(U, V)
    for i in range(n):
        a[slot(i + 1)] = x[i]
    a[c] = 1.0 - x.sum()
    return a, lam


def translation_generators(w):
    """Rigid-shift directions of a field [b][Nz][Ny][Nx]: central differences
    along x, y, z on the periodic grid, in grid units (None for a length-1
    axis).  w(r - d) = w(r) - sum_a d_a t_a(r) + O(d^2)."""
    out = []
    for ax, n in ((3, w.shape[3]), (2, w.shape[2]), (1, w.shape[1])):
        out.append(None if n == 1 else 0.5 * (np.roll(w, -1, axis=ax) - np.roll(w, 1, axis=ax)))
    return out


def remove_translation(wa0, wb0, wa1, wb1):
    """The field update (wa0, wb0) -> (wa1, wb1) with its component along the
    rigid shifts of (wa0, wb0) removed, per instance (least squares over both
    fields: 3x3 normal equations of the generators).  Without it, an
    iteration may drift along the translational zero mode (a converged
    periodic structure is defined only up to a shift), and two runs of
    different arithmetic drift differently."""
    ta, tb = translation_generators(wa0), translation_generators(wb0)
    axes = [k for k in range(3) if ta[k] is not None]
    b = wa0.shape[0]
    da, db = wa1 - wa0, wb1 - wb0
    outa, outb = wa1.copy(), wb1.copy()
    for bi in range(b):
        n = len(axes)
        G = np.empty((n, n))
        c = np.empty(n)
        for i, ai in enumerate(axes):
            c[i] = (ta[ai][bi] * da[bi]).sum() + (tb[ai][bi] * db[bi]).sum()
            for j, aj in enumerate(axes):
                G[i, j] = (ta[ai][bi] * ta[aj][bi]).sum() + (tb[ai][bi] * tb[aj][bi]).sum()
        G += np.eye(n) * (1e-14 * np.abs(np.diag(G)).max() + 1e-300)
        alpha = np.linalg.solve(G, c)
        for i, ai in enumerate(axes):
            outa[bi] -= alpha[i] * ta[ai][bi]
            outb[bi] -= alpha[i] * tb[ai][bi]
    return outa, outb


def converge_loop(wa, wb, p: Params, tol, max_it, mixing="anderson", m=20, lam=0.5,
                  start=1e-2, pin_translation=False):
    """Iterate Free's body (average_value x2, getConc, field update) until
    max(err_max) < tol; returns (wa, wb, pha, phb, Q, iters, err_history).
    pin_translation: each Anderson update without its rigid-shift component
    (remove_translation), as the library's SCFT_FLAG_PIN_TRANSLATION."""
    kdz = kxyzdz_half(p)
    b = wa.shape[0]
    m1 = m + 1
    hw = [None] * m1
    hd = [None] * m1
    G = np.zeros((b, m1, m1))
    count = 0
    errs = []
    it = 0
    pha = phb = Q = None
    while it < max_it:
        it += 1
        wa = average_value(wa)
        wb = average_value(wb)
        cc = get_conc(wa, wb, p, kdz)
        wa, pha, phb, Q = cc.wa, cc.pha, cc.phb, cc.Q
        da, db, emax, erms, ca, cb = residual(wa, wb, pha, phb, p.hAB, p.wcmp)
        errs.append(emax.max())
        if mixing == "simple":
            wa = wa + p.wopt * da
            wb = wb + p.wopt * db
        else:
            c = count % m1
            hist = min(count, m)
            hw[c] = np.concatenate([wa.reshape(b, -1), wb.reshape(b, -1)], axis=1)
            hd[c] = np.concatenate([ca.reshape(b, -1), cb.reshape(b, -1)], axis=1)
            for k in range(hist + 1):
                j = (c - k) % m1
                g = (hd[c] * hd[j]).sum(axis=1)
                G[:, c, j] = g
                G[:, j, c] = g
            new = np.zeros_like(hw[c])
            for bi in range(b):
                a, l = anderson_weights(G[bi], c, hist, m1, emax[bi], start, lam, p.wopt)
                for j in range(m1):
                    if a[j] != 0.0:
                        new[bi] += a[j] * (hw[j][bi] + l * hd[j][bi])
            M = p.M
            wa1 = new[:, :M].reshape(wa.shape)
            wb1 = new[:, M:].reshape(wb.shape)
            if pin_translation:
                wa1, wb1 = remove_translation(wa, wb, wa1, wb1)
            wa, wb = wa1, wb1
            count += 1
        if emax.max() < tol:
            break
    return wa, wb, pha, phb, Q, it, errs
