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


def _noalloc(lib, fin, fout, n, area, wl, z, flags=0, stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    st = ctypes.c_void_p(s.cuda_stream)
    return lib.lp_plain_propagate_field_noalloc(ctypes.c_void_p(fin.data_ptr()),
                                                ctypes.c_void_p(fout.data_ptr()),
                                                n, area, wl, z, flags, st)


def _rel(a, b):
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


@pytest.mark.parametrize("n,area,wl,z", [(256, 0.05, 632e-7, 0.7),
                                         (1024, 0.2, 1064e-7, 3.0)])
def test_noalloc_matches_plain_and_oracle_on_two_calls_in_a_row(n, area, wl, z):
    from lightprop2d_gb300 import _lib as L
    from lightprop2d_gb300 import backend as B
    from oracle import lp_oracle as O
    lib = L.load()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(n)
    g = O.grids(area, n, wl)
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
        # and against the complex128 restatement of the reference's propagate
        _, want = O.propagate(np.fft.fft2(x.cpu().numpy().astype(np.complex128)), g["Kz"], z)
        assert O.rel_l2(y.cpu().numpy(), want) < TOL


def test_noalloc_allocates_no_device_memory():
    from lightprop2d_gb300 import _lib as L
    lib = L.load()
    torch.cuda.set_device(0)
    n = 1024
    x = torch.ones((n, n), dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    L.check(_noalloc(lib, x, y, n, 0.2, 632e-7, 1.0), "warm-up call")
    torch.cuda.synchronize()
    s = torch.cuda.Stream()  # a stream the entry point has never seen
    free0, _ = torch.cuda.mem_get_info()
    with torch.cuda.stream(s):
        L.check(_noalloc(lib, x, y, n, 0.2, 632e-7, 2.0, stream=s), "call on a new stream")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_array():
    from lightprop2d_gb300 import _lib as L
    lib = L.load()
    x = torch.zeros((2048, 2048), dtype=torch.complex64, device="cuda")
    st = _noalloc(lib, x, x, 2048, 0.2, 632e-7, 1.0)
    assert st == L.LP_ERR_UNSUPPORTED_SIZE
    assert b"1024" in lib.lp_last_error()


_FIRST_CALL_IN_CAPTURE = r"""
import ctypes, sys, torch
sys.path.insert(0, sys.argv[1])
from lightprop2d_gb300 import _lib as L
lib = L.load()
torch.cuda.set_device(0)
x = torch.zeros((64, 64), dtype=torch.complex64, device="cuda")
s = torch.cuda.Stream()
g = torch.cuda.CUDAGraph()
with torch.cuda.stream(s):
    g.capture_begin()
    st = lib.lp_plain_propagate_field_noalloc(ctypes.c_void_p(x.data_ptr()),
                                              ctypes.c_void_p(x.data_ptr()), 64, 0.05,
                                              632e-7, 1.0, 0, ctypes.c_void_p(s.cuda_stream))
    g.capture_end()
print(st)
"""


def test_noalloc_first_call_inside_capture_is_refused():
    """In a fresh process the first call is the set-up call: made while its
    stream captures, it returns LP_ERR_NOT_INITIALIZED and leaves the capture
    intact."""
    import os
    import subprocess
    import sys
    from lightprop2d_gb300 import _lib as L
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "-c", _FIRST_CALL_IN_CAPTURE, root],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert int(p.stdout.strip().splitlines()[-1]) == L.LP_ERR_NOT_INITIALIZED
