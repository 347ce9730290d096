"""GB300-native diblock-copolymer SCFT hot path: Python host mirror.

A thin ctypes layer over the C ABI of ``include/scft_capi.h`` (the CUDA
library ``libscft_gb300.so`` built in-tree by ``build.py``).  Method names
follow the reference's C++ API (``average_value``, ``sov_dif_fft``,
``get_conc``, ``phi_w``, ``free``), arrays are float64 numpy arrays shaped
``[batch, Nz, Ny, Nx]``.  There is no CPU fallback: if the library is
missing, loading raises.

The directory name is not a Python identifier; import it with
``load_package()`` from ``__graft_entry__`` (registered as ``scft_gb300``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libscft_gb300.so")

OK = 0
ERR_INVALID_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NO_MEMORY = 1, 2, 3, 4
ERR_NOT_FINITE, ERR_IO, ERR_NO_DEVICE = 5, 6, 7
PREC_FP64, PREC_FP32, PREC_DF = 0, 1, 2
FIELD_WA, FIELD_WB, FIELD_PHA, FIELD_PHB = 0, 1, 2, 3
Q_A, Q_CB, Q_B, Q_CA = 0, 1, 2, 3
MIX_SIMPLE, MIX_ANDERSON, MIX_CONSTRAINED, MIX_CONSTRAINED_EX = 0, 1, 2, 3

# Every symbol include/scft_capi.h declares (checked by the CPU tests).
EXPORTS = [
    "scft_params_default", "scft_grid_supported", "scft_create", "scft_destroy",
    "scft_last_error", "scft_strerror", "scft_get_ns", "scft_set_field", "scft_get_field",
    "scft_average_value", "scft_sov_dif_fft", "scft_set_qint", "scft_get_q", "scft_get_conc",
    "scft_get_Q", "scft_phi_w", "scft_free_energy", "scft_iterate", "scft_free",
    "scft_synchronize", "scft_launch_count", "scft_read_ab_txt", "scft_read_phi_dat",
    "scft_write_pha_dat", "scft_time_iterations", "scft_profile_enable", "scft_profile_read",
    "scft_split_step_noalloc", "scft_noalloc_last_error", "scft_get_residual", "scft_converge",
    "scft_copy_fields", "scft_group_create", "scft_group_destroy", "scft_group_last_error",
    "scft_group_iterate", "scft_group_time_iterations", "scft_group_launch_count",
    "scft_get_schedule", "scft_write_vtk", "scft_convert_pha_to_vtk", "scft_set_target",
    "scft_save_checkpoint", "scft_load_checkpoint", "scft_set_metrics_file",
    "scft_phi_w_constrained", "scft_set_box", "scft_stress", "scft_adjoint",
    "scft_adjoint_checkpoints", "scft_relax_cell", "scft_get_box", "scft_field_device_ptr",
    "scft_get_stream", "scft_copy_q_reference_layout", "scft_selftest_bounded_wait", "scft_spline", "scft_spline_eval",
    "scft_spline_deriv", "scft_spline_integral", "scft_spline_eval_device",
    "scft_shard_plan", "scft_free_shards",
]
FLAG_NO_GRAPH, FLAG_PIPE, FLAG_TWO_STREAMS, FLAG_LOCKSTEP, FLAG_NO_XY = 1, 2, 4, 8, 16
FLAG_AUTOTUNE, FLAG_NO_FUSED_STEPS, FLAG_SIMPSON, FLAG_PIN_TRANSLATION = 32, 64, 128, 256


class ScftParams(C.Structure):
    """Mirror of ``scft_params`` (include/scft_capi.h)."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("hAB", C.c_double), ("fA", C.c_double), ("ds0", C.c_double),
        ("batch", C.c_int), ("precision", C.c_int),
        ("wopt", C.c_double), ("wcmp", C.c_double),
        ("mixing", C.c_int), ("anderson_history", C.c_int), ("anderson_lambda", C.c_double),
        ("device", C.c_int), ("flags", C.c_int), ("anderson_start", C.c_double),
        ("constraint_lambda", C.c_double), ("reserved", C.c_int * 4),
    ]


class ScftError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"scft status {status}: {msg}")
        self.status = status


_lib = None


def load_library(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    lib = C.CDLL(p)
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    sig = {
        "scft_params_default": (C.c_int, [C.POINTER(ScftParams)]),
        "scft_grid_supported": (C.c_int, [C.c_int, C.c_int, C.c_int]),
        "scft_create": (C.c_int, [C.POINTER(ScftParams), C.POINTER(vp)]),
        "scft_destroy": (None, [vp]),
        "scft_last_error": (C.c_char_p, [vp]),
        "scft_strerror": (C.c_char_p, [C.c_int]),
        "scft_get_ns": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "scft_set_field": (C.c_int, [vp, C.c_int, dp]),
        "scft_get_field": (C.c_int, [vp, C.c_int, dp]),
        "scft_average_value": (C.c_int, [vp, C.c_int]),
        "scft_sov_dif_fft": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "scft_set_qint": (C.c_int, [vp, C.c_int, C.c_int]),
        "scft_get_q": (C.c_int, [vp, C.c_int, C.c_int, dp]),
        "scft_get_conc": (C.c_int, [vp]),
        "scft_get_Q": (C.c_int, [vp, dp]),
        "scft_phi_w": (C.c_int, [vp]),
        "scft_free_energy": (C.c_int, [vp, dp]),
        "scft_iterate": (C.c_int, [vp, C.c_int, dp]),
        "scft_free": (C.c_int, [vp, C.c_int, C.c_int, C.c_char_p]),
        "scft_shard_plan": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]),
        "scft_free_shards": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_char_p]),
        "scft_synchronize": (C.c_int, [vp]),
        "scft_launch_count": (C.c_longlong, [vp]),
        "scft_read_ab_txt": (C.c_int, [C.c_char_p, C.POINTER(ScftParams), C.POINTER(C.c_int)]),
        "scft_read_phi_dat": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "scft_write_pha_dat": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "scft_time_iterations": (C.c_int, [vp, C.c_int, dp]),
        "scft_profile_enable": (C.c_int, [vp, C.c_int]),
        "scft_profile_read": (C.c_int, [vp, dp, C.POINTER(C.c_longlong), dp]),
        "scft_split_step_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                              C.c_double, C.c_double, C.c_int, vp, vp, vp, vp]),
        "scft_noalloc_last_error": (C.c_char_p, []),
        "scft_get_residual": (C.c_int, [vp, dp, dp]),
        "scft_converge": (C.c_int, [vp, C.c_double, C.c_int, C.POINTER(C.c_int), dp]),
        "scft_copy_fields": (C.c_int, [vp, vp]),
        "scft_group_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(vp)]),
        "scft_group_destroy": (None, [vp]),
        "scft_group_last_error": (C.c_char_p, [vp]),
        "scft_group_iterate": (C.c_int, [vp, C.c_int]),
        "scft_group_time_iterations": (C.c_int, [vp, C.c_int, dp]),
        "scft_group_launch_count": (C.c_longlong, [vp]),
        "scft_get_schedule": (C.c_int, [vp, C.POINTER(C.c_int), dp]),
        "scft_write_vtk": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_char_p]),
        "scft_convert_pha_to_vtk": (C.c_int, [C.c_char_p, C.c_char_p]),
        "scft_save_checkpoint": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "scft_load_checkpoint": (C.c_int, [vp, C.c_char_p]),
        "scft_set_metrics_file": (C.c_int, [vp, C.c_char_p]),
        "scft_set_target": (C.c_int, [vp, dp]),
        "scft_phi_w_constrained": (C.c_int, [vp, C.c_int, C.c_double]),
        "scft_set_box": (C.c_int, [vp, C.c_double, C.c_double, C.c_double]),
        "scft_get_box": (C.c_int, [vp, dp]),
        "scft_field_device_ptr": (C.c_int, [vp, C.c_int, C.POINTER(dp)]),
        "scft_get_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "scft_copy_q_reference_layout": (C.c_int, [vp, C.c_int, vp]),
        "scft_selftest_bounded_wait": (C.c_int, [C.c_int, C.c_double, C.POINTER(C.c_int)]),
        "scft_spline": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, dp, dp, dp,
                                  dp, dp, C.POINTER(C.c_int)]),
        "scft_spline_eval": (C.c_double, [C.c_int, C.c_double, dp, dp, dp, dp, dp,
                                          C.POINTER(C.c_int)]),
        "scft_spline_deriv": (C.c_double, [C.c_int, C.c_double, dp, dp, dp, dp,
                                           C.POINTER(C.c_int)]),
        "scft_spline_integral": (C.c_double, [C.c_int, C.c_double, dp, dp, dp, dp, dp,
                                              C.POINTER(C.c_int)]),
        "scft_spline_eval_device": (C.c_int, [C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_longlong,
                                              C.c_int, vp]),
        "scft_stress": (C.c_int, [vp, dp]),
        "scft_adjoint": (C.c_int, [vp, dp, dp, dp, dp, dp, dp, C.c_int]),
        "scft_adjoint_checkpoints": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int),
                                               C.POINTER(C.c_longlong)]),
        "scft_relax_cell": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                      C.c_double, C.POINTER(C.c_int), dp, dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def shard_plan(num_scft: int, gpu_n: int):
    """The reference's split of Num_SCFT instances over GPU_N devices
    (init_cuda.cu:312): -> (instances per device, instances not run)."""
    lib = load_library()
    b, nr = C.c_int(), C.c_int()
    st = lib.scft_shard_plan(num_scft, gpu_n, C.byref(b), C.byref(nr))
    if st != OK:
        raise ScftError(st, lib.scft_last_error(None).decode())
    return b.value, nr.value


def free_shards(ctxs, max_it: int, aver_it: int = 10, outdir: str | None = None):
    """Free over contexts holding consecutive instance shards (one per
    device): scft_free_shards."""
    lib = load_library()
    arr = (C.c_void_p * len(ctxs))(*[c.h for c in ctxs])
    st = lib.scft_free_shards(arr, len(ctxs), max_it, aver_it,
                              outdir.encode() if outdir else None)
    if st != OK:
        raise ScftError(st, lib.scft_last_error(ctxs[0].h).decode())


def default_params(**kw) -> ScftParams:
    lib = load_library()
    p = ScftParams()
    lib.scft_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def read_ab_txt(path: str):
    """Parse ``ab.txt`` (init.cpp:81-94) -> (ScftParams, intag)."""
    lib = load_library()
    p = ScftParams()
    tag = C.c_int(0)
    st = lib.scft_read_ab_txt(path.encode(), C.byref(p), C.byref(tag))
    if st != OK:
        raise ScftError(st, lib.scft_last_error(None).decode())
    return p, tag.value


def convert_pha_to_vtk(pha_path: str, vtk_path: str):
    """The reference's pha file -> VTK converter (vtk.c)."""
    lib = load_library()
    st = lib.scft_convert_pha_to_vtk(pha_path.encode(), vtk_path.encode())
    if st != OK:
        raise ScftError(st, lib.scft_last_error(None).decode())


class Spline:
    """Cubic interpolating spline (the reference's spline.c: spline, seval,
    deriv, sinteg), coefficients from the library's scft_spline."""

    def __init__(self, x, y, end1: int = 0, end2: int = 0, slope1: float = 0.0,
                 slope2: float = 0.0):
        self.lib = load_library()
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        n = self.n = len(self.x)
        self.b, self.c, self.d = np.zeros(n), np.zeros(n), np.zeros(n)
        flag = C.c_int()
        st = self.lib.scft_spline(n, end1, end2, slope1, slope2, _dptr(self.x), _dptr(self.y),
                                  _dptr(self.b), _dptr(self.c), _dptr(self.d), C.byref(flag))
        if st != OK:
            raise ScftError(st, "scft_spline")
        self.iflag = flag.value
        self.last = C.c_int(0)

    def _args(self):
        return _dptr(self.x), _dptr(self.y), _dptr(self.b), _dptr(self.c), _dptr(self.d)

    def __call__(self, u: float) -> float:
        x, y, b, c, d = self._args()
        return self.lib.scft_spline_eval(self.n, u, x, y, b, c, d, C.byref(self.last))

    def deriv(self, u: float) -> float:
        x, _, b, c, d = self._args()
        return self.lib.scft_spline_deriv(self.n, u, x, b, c, d, C.byref(self.last))

    def integral(self, u: float) -> float:
        x, y, b, c, d = self._args()
        return self.lib.scft_spline_integral(self.n, u, x, y, b, c, d, C.byref(self.last))

    def eval_device(self, u, mode: int = 0):
        """Batched evaluation on the GPU: u a CUDA float64 tensor -> tensor
        (mode 0 value, 1 derivative, 2 integral from x[0])."""
        import torch
        dev = u.device
        coef = [torch.as_tensor(a, device=dev) for a in (self.x, self.y, self.b, self.c, self.d)]
        out = torch.empty_like(u)
        torch.cuda.synchronize(dev)
        st = self.lib.scft_spline_eval_device(self.n, *[t.data_ptr() for t in coef], u.data_ptr(),
                                              out.data_ptr(), u.numel(), mode, None)
        torch.cuda.synchronize(dev)
        if st != OK:
            raise ScftError(st, "scft_spline_eval_device")
        return out


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Context:
    """One device context: ``batch`` instances of one grid (scft_ctx)."""

    def __init__(self, params: ScftParams | None = None, **kw):
        self.lib = load_library()
        self.params = params if params is not None else default_params(**kw)
        if params is not None:
            for k, v in kw.items():
                setattr(self.params, k, v)
        h = C.c_void_p()
        st = self.lib.scft_create(C.byref(self.params), C.byref(h))
        if st != OK:
            raise ScftError(st, self.lib.scft_last_error(None).decode())
        self.h = h
        a, b = C.c_int(), C.c_int()
        self.lib.scft_get_ns(self.h, C.byref(a), C.byref(b))
        self.NsA, self.dNsB = a.value, b.value
        p = self.params
        self.shape = (p.batch, p.nz, p.ny, p.nx)

    # -- plumbing
    def _ck(self, st):
        if st != OK:
            raise ScftError(st, self.lib.scft_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.scft_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- fields
    def set_field(self, field: int, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        self._ck(self.lib.scft_set_field(self.h, field, _dptr(a)))

    def get_field(self, field: int) -> np.ndarray:
        out = np.empty(self.shape)
        self._ck(self.lib.scft_get_field(self.h, field, _dptr(out)))
        return out

    def set_w(self, wa, wb):
        self.set_field(FIELD_WA, wa)
        self.set_field(FIELD_WB, wb)

    @property
    def wa(self):
        return self.get_field(FIELD_WA)

    @property
    def wb(self):
        return self.get_field(FIELD_WB)

    @property
    def pha(self):
        return self.get_field(FIELD_PHA)

    @property
    def phb(self):
        return self.get_field(FIELD_PHB)

    # -- hot path (reference API names)
    def average_value(self, field: int):
        self._ck(self.lib.scft_average_value(self.h, field))

    def set_qint(self, q: int = -1, s: int = 0):
        self._ck(self.lib.scft_set_qint(self.h, q, s))

    def sov_dif_fft(self, q: int, w_field: int, ns: int, sign: int):
        self._ck(self.lib.scft_sov_dif_fft(self.h, q, w_field, ns, sign))

    def get_q(self, q: int, s: int) -> np.ndarray:
        out = np.empty(self.shape)
        self._ck(self.lib.scft_get_q(self.h, q, s, _dptr(out)))
        return out

    def get_conc(self):
        self._ck(self.lib.scft_get_conc(self.h))

    def Q(self) -> np.ndarray:
        out = np.empty(self.shape[0])
        self._ck(self.lib.scft_get_Q(self.h, _dptr(out)))
        return out

    def phi_w(self):
        self._ck(self.lib.scft_phi_w(self.h))

    def free_energy(self) -> np.ndarray:
        out = np.empty((self.shape[0], 5))
        self._ck(self.lib.scft_free_energy(self.h, _dptr(out)))
        return out

    def iterate(self, n: int, with_energy: bool = False):
        if with_energy:
            out = np.empty((self.shape[0], 5))
            self._ck(self.lib.scft_iterate(self.h, n, _dptr(out)))
            return out
        self._ck(self.lib.scft_iterate(self.h, n, None))
        return None

    def free(self, max_it: int, aver_it: int = 10, outdir: str | None = None):
        self._ck(self.lib.scft_free(self.h, max_it, aver_it,
                                    outdir.encode() if outdir else None))

    def synchronize(self):
        self._ck(self.lib.scft_synchronize(self.h))

    def launch_count(self) -> int:
        return int(self.lib.scft_launch_count(self.h))

    def schedule(self):
        """-> (SCFT_FLAG_* bits of the march schedule in use, autotuned march ms or 0)."""
        f, ms = C.c_int(), C.c_double()
        self._ck(self.lib.scft_get_schedule(self.h, C.byref(f), C.byref(ms)))
        return f.value, ms.value

    def residual(self):
        """-> (err_max[batch], err_rms[batch]) of the last field update."""
        mx, rms = np.empty(self.shape[0]), np.empty(self.shape[0])
        self._ck(self.lib.scft_get_residual(self.h, _dptr(mx), _dptr(rms)))
        return mx, rms

    def converge(self, tol: float, max_it: int):
        """Iterate to max-norm residual < tol -> (iterations, free energy [batch, 5])."""
        it = C.c_int()
        out = np.empty((self.shape[0], 5))
        self._ck(self.lib.scft_converge(self.h, tol, max_it, C.byref(it), _dptr(out)))
        return it.value, out

    def copy_fields_from(self, other: "Context"):
        self._ck(self.lib.scft_copy_fields(self.h, other.h))

    def time_iterations(self, n: int) -> float:
        """Device milliseconds of n SCF iterations (events on the library's stream)."""
        ms = C.c_double()
        self._ck(self.lib.scft_time_iterations(self.h, n, C.byref(ms)))
        return ms.value

    def profile_enable(self, reserve_marches: int):
        self._ck(self.lib.scft_profile_enable(self.h, reserve_marches))

    def profile_read(self):
        """-> (summed march milliseconds, number of marches, point-steps)."""
        ms, n, ps = C.c_double(), C.c_longlong(), C.c_double()
        self._ck(self.lib.scft_profile_read(self.h, C.byref(ms), C.byref(n), C.byref(ps)))
        return ms.value, n.value, ps.value

    def read_phi_dat(self, path: str, inst: int = 0):
        self._ck(self.lib.scft_read_phi_dat(self.h, path.encode(), inst))

    def write_pha_dat(self, path: str, inst: int = 0):
        self._ck(self.lib.scft_write_pha_dat(self.h, path.encode(), inst))

    def write_vtk(self, path: str, inst: int = 0, source: str = "pha.dat"):
        """phiA - phiB of one instance as the reference converter's VTK file."""
        self._ck(self.lib.scft_write_vtk(self.h, path.encode(), inst, source.encode()))

    def save_checkpoint(self, path: str, with_history: bool = True):
        """Binary FP64 checkpoint (fields, and the Anderson history when kept)
        for an exact resume."""
        self._ck(self.lib.scft_save_checkpoint(self.h, str(path).encode(), int(with_history)))

    def load_checkpoint(self, path: str):
        """Restore a checkpoint written by save_checkpoint (same grid and batch)."""
        self._ck(self.lib.scft_load_checkpoint(self.h, str(path).encode()))

    def set_metrics_file(self, path):
        """JSON-lines progress reports of free() to `path` (None: off)."""
        self._ck(self.lib.scft_set_metrics_file(self.h, str(path).encode() if path else None))

    def set_target(self, pha_target: np.ndarray):
        """Target phiA of the constrained updates ([batch, Nz, Ny, Nx] or [Nz, Ny, Nx])."""
        a = np.ascontiguousarray(np.broadcast_to(pha_target, self.shape), dtype=np.float64)
        self._ck(self.lib.scft_set_target(self.h, _dptr(a)))

    def phi_w_constrained(self, ex: bool = False, lam: float = 0.0):
        """One phi_w_constrained (ex False) or phi_w_constrainedEx (ex True) update."""
        self._ck(self.lib.scft_phi_w_constrained(self.h, int(bool(ex)), lam))

    def set_box(self, lx: float, ly: float, lz: float):
        self._ck(self.lib.scft_set_box(self.h, lx, ly, lz))
        self.params.lx, self.params.ly, self.params.lz = lx, ly, lz

    def field_view(self, field: int):
        """A torch tensor over the device memory of a field (no copy),
        shape [batch, Nz, Ny, Nx], float64.  Synchronise (``synchronize()`` /
        ``torch.cuda.synchronize()``) between library calls and torch work."""
        import torch
        dp_out = C.POINTER(C.c_double)()
        self._ck(self.lib.scft_field_device_ptr(self.h, field, C.byref(dp_out)))
        addr = C.cast(dp_out, C.c_void_p).value

        class _Iface:
            __cuda_array_interface__ = {"shape": tuple(self.shape), "typestr": "<f8",
                                        "data": (addr, False), "version": 3, "strides": None}
        return torch.as_tensor(_Iface(), device=f"cuda:{self.params.device}")

    def box(self) -> np.ndarray:
        out = np.empty(3)
        self._ck(self.lib.scft_get_box(self.h, _dptr(out)))
        return out

    def stress(self) -> np.ndarray:
        """-d ln Q / dL [batch, 3] of the propagators of the last getConc."""
        out = np.empty((self.shape[0], 3))
        self._ck(self.lib.scft_stress(self.h, _dptr(out)))
        return out

    def adjoint(self, pha_bar=None, phb_bar=None, Q_bar=None, want_L: bool = True,
                checkpoint_every: int = 0):
        """Vector-Jacobian product of getConc at the current fields:
        -> (wa_bar, wb_bar, L_bar[batch, 3] or None)."""
        def seed(a):
            if a is None:
                return None
            return np.ascontiguousarray(np.broadcast_to(a, self.shape), dtype=np.float64)
        pa, pb = seed(pha_bar), seed(phb_bar)
        qb = None if Q_bar is None else np.ascontiguousarray(
            np.broadcast_to(Q_bar, (self.shape[0],)), dtype=np.float64)
        wa_bar, wb_bar = np.empty(self.shape), np.empty(self.shape)
        L_bar = np.empty((self.shape[0], 3)) if want_L else None
        p = lambda a: None if a is None else _dptr(a)
        self._ck(self.lib.scft_adjoint(self.h, p(pa), p(pb), p(qb), _dptr(wa_bar), _dptr(wb_bar),
                                       p(L_bar), checkpoint_every))
        return wa_bar, wb_bar, L_bar

    def relax_cell(self, axes_mask: int = 7, tol_w: float = 1e-8, tol_stress: float = 1e-6,
                   max_outer: int = 50, max_inner: int = 5000, step0: float = 1.0):
        """Unit-cell relaxation -> (rounds, final stress [3], free energy [5]);
        the context keeps the relaxed box (``box()``)."""
        n = C.c_int()
        sig, fe = np.empty(3), np.empty(5)
        self._ck(self.lib.scft_relax_cell(self.h, axes_mask, tol_w, tol_stress, max_outer,
                                          max_inner, step0, C.byref(n), _dptr(sig), _dptr(fe)))
        return n.value, sig, fe

    def adjoint_checkpoints(self, checkpoint_every: int = 0):
        """-> (propagator slices held by the adjoint, bytes)."""
        n, b = C.c_int(), C.c_longlong()
        self._ck(self.lib.scft_adjoint_checkpoints(self.h, checkpoint_every, C.byref(n),
                                                   C.byref(b)))
        return n.value, b.value


class Group:
    """Heterogeneous batched sweep over several contexts (scft_group): one
    CUDA-graph launch per iteration advances every member."""

    def __init__(self, members):
        self.lib = load_library()
        self.members = list(members)          # keep the contexts alive
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h = C.c_void_p()
        st = self.lib.scft_group_create(arr, len(self.members), C.byref(h))
        if st != OK:
            raise ScftError(st, self.lib.scft_last_error(None).decode())
        self.h = h

    def _ck(self, st):
        if st != OK:
            raise ScftError(st, self.lib.scft_group_last_error(self.h).decode())

    def iterate(self, n: int):
        self._ck(self.lib.scft_group_iterate(self.h, n))

    def time_iterations(self, n: int) -> float:
        ms = C.c_double()
        self._ck(self.lib.scft_group_time_iterations(self.h, n, C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        return int(self.lib.scft_group_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.scft_group_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
