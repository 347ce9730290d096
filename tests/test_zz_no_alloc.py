"""scft_split_step_noalloc: the split step for callers that cannot allocate
device memory where they advance a propagator (a framework that owns every
device allocation through its own pool, or a latency-critical loop that
cannot take cudaMalloc's implicit synchronisation).  The caller passes its own
q_in, W and q_out; scratch is the library's static device array.

Checked through the C ABI on two calls in a row against the CPU oracle's split
step (orc.sov_dif_fft) and against the existing entry point (scft_sov_dif_fft,
which allocates at context creation), with the FP32 tolerance of the other
parity tests.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-5


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


GRIDS = [(64, 32, 32, 3.8, 3.0, 3.0),    # register kernels
         (16, 12, 8, 4.0, 3.0, 2.5),     # generic Stockham kernels
         (16, 16, 1, 4.0, 4.0, 2.0)]     # a length-1 axis: its constant factor folds into x


def step_twice(pkg, grid, ds0, batch, wa, q0, stream=None):
    """Two no-allocation steps in a row from q0 (FP64 host array); returns
    both outputs as FP64 host arrays."""
    import torch
    nx, ny, nz, lx, ly, lz = grid
    lib = pkg.load_library()
    dev = torch.device("cuda:0")
    W = torch.from_numpy(np.exp(-wa.astype(np.float32) * np.float32(ds0 / 2))).to(dev)
    q = torch.from_numpy(q0.astype(np.float32)).to(dev)
    outs = [torch.empty_like(q), torch.empty_like(q)]
    torch.cuda.synchronize()
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    for k in range(2):
        src = q if k == 0 else outs[0]
        st = lib.scft_split_step_noalloc(nx, ny, nz, lx, ly, lz, ds0, batch,
                                         C.c_void_p(src.data_ptr()), C.c_void_p(W.data_ptr()),
                                         C.c_void_p(outs[k].data_ptr()), handle)
        assert st == 0, lib.scft_noalloc_last_error().decode()
    torch.cuda.synchronize()
    return [o.double().cpu().numpy() for o in outs]


@pytest.mark.parametrize("grid", GRIDS, ids=["register", "generic", "length1"])
def test_noalloc_matches_oracle_and_existing_entry_point(pkg, orc, grid):
    from scft_gb300 import fields
    nx, ny, nz, lx, ly, lz = grid
    batch, ds0 = 2, 0.02
    wa, _ = fields.gyroid(nx, ny, nz, lx, ly, lz, 18.0, seed=5, batch=batch)
    p = orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=18.0, fA=0.36, ds0=ds0,
                   batch=batch)
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=18.0, fA=0.36, ds0=ds0,
                     batch=batch, precision=pkg.PREC_FP32) as ctx:
        ctx.set_w(wa, np.zeros_like(wa))
        ctx.set_qint(-1)
        ctx.sov_dif_fft(pkg.Q_A, pkg.FIELD_WA, 3, +1)          # existing entry point
        ref = [ctx.get_q(pkg.Q_A, s) for s in range(4)]
    # the oracle, stepped from the same (FP32-rounded) input slice
    q0 = ref[1].astype(np.float32).astype(np.float64)
    orc_q = orc.sov_dif_fft(q0, wa, 2, +1, p)
    outs = step_twice(pkg, grid, ds0, batch, wa, ref[1])
    assert rel(outs[0], orc_q[:, 1]) < TOL
    assert rel(outs[1], orc_q[:, 2]) < TOL
    assert rel(outs[0], ref[2]) < TOL
    assert rel(outs[1], ref[3]) < TOL


def test_noalloc_on_a_caller_stream_allocates_nothing(pkg, orc):
    """A non-default stream, and no change of the device's free memory across
    calls once the first call on the device has looked up its array."""
    import torch
    from scft_gb300 import fields
    grid = GRIDS[0]
    nx, ny, nz, lx, ly, lz = grid
    batch, ds0 = 1, 0.02
    wa, _ = fields.gyroid(nx, ny, nz, lx, ly, lz, 18.0, seed=6, batch=batch)
    q0 = np.ones_like(wa)
    p = orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=18.0, fA=0.36, ds0=ds0,
                   batch=batch)
    orc_q = orc.sov_dif_fft(q0, wa, 2, +1, p)
    stream = torch.cuda.Stream()
    step_twice(pkg, grid, ds0, batch, wa, q0)                 # first call: set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    outs = step_twice(pkg, grid, ds0, batch, wa, q0, stream=stream)
    free1, _ = torch.cuda.mem_get_info()
    assert rel(outs[0], orc_q[:, 1]) < TOL
    assert rel(outs[1], orc_q[:, 2]) < TOL
    # torch allocated its own input/output buffers between the readings only
    # from its cache (already reserved by the first round), so the device's
    # free memory is unchanged
    assert free1 == free0


def test_noalloc_ignores_an_earlier_unrelated_error(pkg, orc):
    """A failed CUDA runtime call before the step (here: selecting a device
    that does not exist, which leaves the runtime's last-error state set on
    this host thread) must not make a valid no-allocation call fail."""
    from scft_gb300 import fields
    lib = pkg.load_library()
    t = C.c_int(0)
    assert lib.scft_selftest_bounded_wait(100000, 1.0, C.byref(t)) == pkg.ERR_NO_DEVICE
    grid = GRIDS[1]
    nx, ny, nz, lx, ly, lz = grid
    wa, _ = fields.gyroid(nx, ny, nz, lx, ly, lz, 18.0, seed=7, batch=1)
    p = orc.Params(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=18.0, fA=0.36, ds0=0.02,
                   batch=1)
    q0 = np.ones_like(wa)
    outs = step_twice(pkg, grid, 0.02, 1, wa, q0)
    assert rel(outs[1], orc.sov_dif_fft(q0, wa, 2, +1, p)[:, 2]) < TOL


def test_noalloc_rejects_oversize(pkg):
    lib = pkg.load_library()
    st = lib.scft_split_step_noalloc(128, 128, 128, 4.0, 4.0, 4.0, 0.01, 2, C.c_void_p(16),
                                     C.c_void_p(16), C.c_void_p(16), None)
    assert st == pkg.ERR_INVALID_ARG
    assert b"exceeds the no-allocation maximum" in lib.scft_noalloc_last_error()
    # more instances than a launch grid holds (each a tiny 2x2x1 grid: 4 points)
    st = lib.scft_split_step_noalloc(2, 2, 1, 1.0, 1.0, 1.0, 0.01, 65536, C.c_void_p(16),
                                     C.c_void_p(16), C.c_void_p(16), None)
    assert st == pkg.ERR_INVALID_ARG
    assert b"65535" in lib.scft_noalloc_last_error()
