"""GPU: lp_plain_propagate_field_noalloc, the allocation-free unfused propagate.

It exists for callers that cannot call cudaMalloc while running (a host
application that reserved nearly all device memory for its own pool, or a
real-time loop that forbids device allocation after start-up).  Its H grid is
a fixed 1024^2 device array instead of lp_plain_propagate_field's per-stream
cudaMalloc'd grid.  This file is collected last so that a run that stops at
the first failure has already run every other test; it also passes alone.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-5  # the relative-L2 bar every parity test uses


def _noalloc(lib, fin, fout, n, area, wl, z, flags=0):
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.lp_plain_propagate_field_noalloc(ctypes.c_void_p(fin.data_ptr()),
                                                ctypes.c_void_p(fout.data_ptr()),
                                                n, area, wl, z, flags, st)


def _rel(a, b):
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


@pytest.mark.parametrize("n,area,wl,z", [(256, 0.05, 632e-7, 0.7),
                                         (1024, 0.2, 1064e-7, 3.0)])
def test_noalloc_matches_plain_on_two_calls_in_a_row(n, area, wl, z):
    from lightprop2d_gb300 import _lib as L
    from lightprop2d_gb300 import backend as B
    lib = L.load()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(n)
    outs, ins = [], []
    for _ in range(2):  # two calls in a row share the static H grid
        x = torch.as_tensor(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)),
                            dtype=torch.complex64, device="cuda")
        y = torch.empty_like(x)
        L.check(_noalloc(lib, x, y, n, area, wl, z), "lp_plain_propagate_field_noalloc")
        ins.append(x)
        outs.append(y)
    for x, y in zip(ins, outs):
        ref = B.plain_propagate_field(x, area, wl, z)
        torch.cuda.synchronize()
        assert _rel(y, ref) < TOL


def test_noalloc_rejects_sizes_beyond_its_array():
    from lightprop2d_gb300 import _lib as L
    lib = L.load()
    x = torch.zeros((2048, 2048), dtype=torch.complex64, device="cuda")
    st = _noalloc(lib, x, x, 2048, 0.2, 632e-7, 1.0)
    assert st == L.LP_ERR_UNSUPPORTED_SIZE
    assert b"1024" in lib.lp_last_error()
