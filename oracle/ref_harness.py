"""ctypes wrapper of oracle/_ref/libscft_ref_harness.so (TEST INFRASTRUCTURE
ONLY): the reference's own kernels (oracle/_ref/ref_kernels.cubin, compiled
unchanged from the reference sources) driven in the reference's host order
with cuFFT.  Used by tests/ and tests/golden/make_ref_golden.py."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "libscft_ref_harness.so")
CUBIN = os.path.join(REF_DIR, "ref_kernels.cubin")


def available() -> bool:
    return os.path.exists(LIB) and os.path.exists(CUBIN)


class RefSolver:
    """One reference instance set (batch instances of one grid) on GPU 0."""

    def __init__(self, nx, ny, nz, lx, ly, lz, hAB, fA, ds0, batch=1):
        self.lib = C.CDLL(LIB)
        L = self.lib
        dp = C.POINTER(C.c_double)
        L.ref_last_error.restype = C.c_char_p
        L.ref_open.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                               C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        for n in ("ref_set_field", "ref_get_field"):
            getattr(L, n).argtypes = [C.c_int, dp]
        L.ref_get_Q.argtypes = [dp]
        L.ref_get_q.argtypes = [C.c_int, C.c_int, dp]
        L.ref_average_value.argtypes = [C.c_int]
        L.ref_iterate.argtypes = [C.c_int, dp]
        L.ref_time_iterations.argtypes = [C.c_int, dp]
        L.ref_get_ns.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_set_target.argtypes = [dp]
        L.ref_phi_w_constrained.argtypes = [C.c_int, C.c_double]
        self._ck(L.ref_open(CUBIN.encode(), nx, ny, nz, lx, ly, lz, hAB, fA, ds0, batch))
        a, b = C.c_int(), C.c_int()
        L.ref_get_ns(C.byref(a), C.byref(b))
        self.NsA, self.dNsB = a.value, b.value
        self.shape = (batch, nz, ny, nx)

    def _ck(self, rc):
        if rc != 0:
            raise RuntimeError("reference harness: " + self.lib.ref_last_error().decode())

    @staticmethod
    def _p(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def set_field(self, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        self._ck(self.lib.ref_set_field(which, self._p(a)))

    def get_field(self, which):
        out = np.empty(self.shape)
        self._ck(self.lib.ref_get_field(which, self._p(out)))
        return out

    def set_w(self, wa, wb):
        self.set_field(0, wa)
        self.set_field(1, wb)

    def Q(self):
        out = np.empty(self.shape[0])
        self._ck(self.lib.ref_get_Q(self._p(out)))
        return out

    def get_q(self, which, s):
        out = np.empty(self.shape)
        self._ck(self.lib.ref_get_q(which, s, self._p(out)))
        return out

    def average_value(self, which):
        self._ck(self.lib.ref_average_value(which))

    def get_conc(self):
        self._ck(self.lib.ref_get_conc())

    def phi_w(self):
        self._ck(self.lib.ref_phi_w())

    def set_target(self, pha_target):
        a = np.ascontiguousarray(pha_target, dtype=np.float64).reshape(self.shape)
        self._ck(self.lib.ref_set_target(self._p(a)))

    def phi_w_constrained(self, ex=False, lam=0.0):
        self._ck(self.lib.ref_phi_w_constrained(int(bool(ex)), C.c_double(lam)))

    def iterate(self, n, with_energy=True):
        out = np.empty((self.shape[0], 5))
        self._ck(self.lib.ref_iterate(n, self._p(out) if with_energy else None))
        return out if with_energy else None

    def set_q_mode(self, mode):
        """1 (default): Q from the FP64 sum of the reference's own qB slice;
        0: the value of the reference's cal_ql kernel (which races)."""
        self.lib.ref_set_q_mode(C.c_int(mode))

    def ql_raw(self):
        out = np.empty(self.shape[0])
        self.lib.ref_get_ql_raw(self._p(out))
        return out

    def cal_ql_repeat(self, n):
        out = np.empty(n)
        self._ck(self.lib.ref_cal_ql_repeat(C.c_int(n), self._p(out)))
        return out

    def time_iterations(self, n):
        ms = C.c_double()
        self._ck(self.lib.ref_time_iterations(n, C.byref(ms)))
        return ms.value

    def close(self):
        self.lib.ref_close()
