"""scft_split_step_noalloc: the split step for callers that cannot allocate
device memory (a framework that owns every device allocation through its own
pool, code running during CUDA-graph stream capture, latency-critical loops
that cannot take cudaMalloc's implicit synchronisation).  The caller passes
its own q_in, W and q_out; scratch is the library's static device array.

Checked through the C ABI against the existing entry point (scft_sov_dif_fft,
which allocates at context creation) on two calls in a row, with the FP32
tolerance of the other parity tests.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-5


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("grid", [(64, 32, 32, 3.8, 3.0, 3.0),    # register kernels
                                  (16, 12, 8, 4.0, 3.0, 2.5)])    # generic Stockham kernels
def test_noalloc_matches_existing_entry_point(pkg, grid):
    import torch
    from scft_gb300 import fields
    nx, ny, nz, lx, ly, lz = grid
    batch, ds0 = 2, 0.02
    wa, wb = fields.gyroid(nx, ny, nz, lx, ly, lz, 18.0, seed=5, batch=batch)
    with pkg.Context(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, hAB=18.0, fA=0.36, ds0=ds0,
                     batch=batch, precision=pkg.PREC_FP32) as ctx:
        ctx.set_w(wa, wb)
        ctx.set_qint(-1)
        ctx.sov_dif_fft(pkg.Q_A, pkg.FIELD_WA, 3, +1)          # existing entry point
        ref = [ctx.get_q(pkg.Q_A, s) for s in range(4)]
    lib = pkg.load_library()
    dev = torch.device("cuda:0")
    W = torch.from_numpy(np.exp(-wa.astype(np.float32) * np.float32(ds0 / 2))).to(dev)
    q = torch.from_numpy(ref[1].astype(np.float32)).to(dev)
    outs = [torch.empty_like(q), torch.empty_like(q)]
    torch.cuda.synchronize()
    for k in range(2):                                        # two calls in a row
        src = q if k == 0 else outs[0]
        st = lib.scft_split_step_noalloc(nx, ny, nz, lx, ly, lz, ds0, batch,
                                         C.c_void_p(src.data_ptr()), C.c_void_p(W.data_ptr()),
                                         C.c_void_p(outs[k].data_ptr()), None)
        assert st == 0, lib.scft_noalloc_last_error().decode()
    torch.cuda.synchronize()
    assert rel(outs[0].double().cpu().numpy(), ref[2]) < TOL
    assert rel(outs[1].double().cpu().numpy(), ref[3]) < TOL


def test_noalloc_rejects_oversize(pkg):
    lib = pkg.load_library()
    st = lib.scft_split_step_noalloc(128, 128, 128, 4.0, 4.0, 4.0, 0.01, 2, C.c_void_p(16),
                                     C.c_void_p(16), C.c_void_p(16), None)
    assert st == pkg.ERR_INVALID_ARG
    assert b"exceeds the no-allocation maximum" in lib.scft_noalloc_last_error()
