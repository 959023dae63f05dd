"""GPU: grid sizes that are not powers of two (the reference accepts any
npoints).  They run as Bluestein transforms over the power-of-two kernels
(lp_bluestein.cu): the reference's own runs at npoints 100 and 75 (golden
vectors), the oracle at other sizes (odd, even, and up to 3000, whose work
grid is 8192^2), the adjoint identity, beam moments, and the capture rule."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm = O.um, O.nm, O.mm
TOL = 1e-5


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy() if isinstance(t, torch.Tensor) else t


@pytest.fixture(scope="module")
def lp():
    import lightprop2d_gb300 as lp
    return lp


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)


@pytest.mark.parametrize("bits", [64, 128])
@pytest.mark.parametrize("n,tag", [(100, "np100"), (75, "np75")])
def test_beam2d_against_the_reference_run(lp, golden, n, tag, bits):
    tol = TOL if bits == 64 else 1e-11
    b = lp.Beam2D(1 * mm, n, 632 * nm, init_field=golden[f"{tag}_in"], complex_bits=bits)
    b.lens(5.0)
    b.propagate(0.3)
    assert O.rel_l2(H(b.field), golden[f"{tag}_lens_prop_field"]) < tol
    assert O.rel_l2(H(b.spectrum), golden[f"{tag}_lens_prop_spectrum"]) < tol
    b.coordinate_filter(f_gen=lp.round_hole, fargs=(300 * um,))
    b.spectral_filter(f_gen=lp.gaussian_beam, fargs=(1, 2e4))
    b.propagate(0.5)
    assert O.rel_l2(H(b.field), golden[f"{tag}_filt_prop_field"]) < tol
    ip = b.iprofile
    want = golden[f"{tag}_filt_prop_iprofile"]
    assert np.linalg.norm(ip - want) / np.linalg.norm(want) < tol
    assert b.z == golden[f"{tag}_z"]


@pytest.mark.parametrize("n", [3, 7, 12, 75, 100, 1000, 2047, 3000])
def test_fft2_and_ifft2(n):
    from lightprop2d_gb300 import backend as B
    x = _rand(n, n)
    t = torch.as_tensor(x, device="cuda")
    f = B.fft2(t)
    assert O.rel_l2(H(f), np.fft.fft2(x.astype(np.complex128))) < TOL
    back = B.ifft2(f)
    assert O.rel_l2(H(back), x) < TOL


@pytest.mark.parametrize("n,area,z", [(96, 0.05, 0.7), (75, 0.03, 0.2), (1000, 0.2, 2.0),
                                      (3000, 0.3, 5.0)])
def test_propagate_field_with_lens_kmask_and_iprofile(n, area, z):
    from lightprop2d_gb300 import backend as B
    wl = 632 * nm
    x = _rand(n, 2 * n)
    rng = np.random.default_rng(3)
    km = rng.uniform(0.5, 1.0, size=(n, n)).astype(np.float32)
    g = O.grids(area, n, wl)
    xr = x.astype(np.complex128) * O.lens_phase(g["X"], g["Y"], g["k0"], 7.0)
    spec = O.fft2(xr) * km
    spec_z, want = O.propagate(spec, g["Kz"], z)
    t = torch.as_tensor(x, device="cuda")
    s_out = torch.empty_like(t)
    ip = torch.empty((n, n), dtype=torch.float32, device="cuda")
    got = B.propagate_field(t, area, wl, z, spectrum_out=s_out, iprofile_out=ip, lens_f=7.0,
                            kmask=torch.as_tensor(km, device="cuda"))
    assert O.rel_l2(H(got), want) < TOL
    assert O.rel_l2(H(s_out), spec_z) < TOL
    assert np.linalg.norm(H(ip) - np.abs(want) ** 2) / np.linalg.norm(np.abs(want) ** 2) < TOL


def test_spectrum_state_propagate(lp):
    n, area, wl = 1000, 0.2, 1064 * nm
    f0 = O.gaussian(n, area, 1.0, 200 * um)
    b = lp.Beam2D(area, n, wl, init_field=f0, complex_bits=64)
    o = O.OracleBeam(area, n, wl, init_field=f0)
    for dz in (0.5, 1.5, 3.0):
        b.propagate(dz)
        o.propagate(dz)
        assert O.rel_l2(H(b.field), o.field) < TOL
    assert O.rel_l2(H(b.spectrum), o.spectrum) < TOL


def test_adjoint_identity_odd_size():
    """<P u, v> = <u, P^H v> for the fused operator with a lens and a phase
    mask at an odd size."""
    from lightprop2d_gb300 import _lib as L
    from lightprop2d_gb300 import backend as B
    n, area, wl, z = 125, 0.05, 632 * nm, 0.4
    u = torch.as_tensor(_rand(n, 11), device="cuda")
    v = torch.as_tensor(_rand(n, 12), device="cuda")
    ph = torch.as_tensor(np.random.default_rng(4).uniform(0, 6.3, (n, n)).astype(np.float32),
                         device="cuda")
    pu = B.propagate_field(u, area, wl, z, lens_f=3.0, xmask=ph, xmask_phase=True)
    phv = B.propagate_field(v, area, wl, z, lens_f=3.0, xmask=ph, xmask_phase=True,
                            flags=L.LP_FLAG_ADJOINT)
    a = torch.vdot(v.flatten().to(torch.complex128), pu.flatten().to(torch.complex128))
    b = torch.vdot(phv.flatten().to(torch.complex128), u.flatten().to(torch.complex128))
    assert abs(complex(a) - complex(b)) < 1e-5 * abs(complex(a))


def test_beam_moments_even_size_and_odd_refused(lp):
    n, area = 1000, 0.2
    f = O.gaussian(n, area, 1.0, 150 * um)
    f = np.roll(f, (37, -120), axis=(0, 1))
    b = lp.Beam2D(area, n, 632 * nm, init_field=f, complex_bits=64)
    d4 = b.D4sigma
    d4r = O.d4sigma(f, b.dL)
    assert abs(d4[0] - d4r[0]) < 1e-5 * d4r[0] and abs(d4[1] - d4r[1]) < 1e-5 * d4r[1]
    c = b.centroid
    cr = O.centroid(f, b.dL)
    assert abs(c[0] - cr[0]) < 1e-6 * area and abs(c[1] - cr[1]) < 1e-6 * area
    odd = lp.Beam2D(area, 75, 632 * nm, init_field=np.ones((75, 75)), complex_bits=64)
    with pytest.raises(ValueError):
        odd.D4sigma  # the reference's mgrid does not match an odd grid either


_FIRST_TRANSFORM_IN_CAPTURE = r"""
import ctypes, sys, torch
sys.path.insert(0, sys.argv[1])
from lightprop2d_gb300 import _lib as L
lib = L.load()
torch.cuda.set_device(0)
L.check(lib.lp_init(0), "init")
x = torch.zeros((77, 77), dtype=torch.complex64, device="cuda")
s = torch.cuda.Stream()
g = torch.cuda.CUDAGraph()
with torch.cuda.stream(s):
    g.capture_begin()
    st = lib.lp_fft2(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()), 77, 0,
                     ctypes.c_void_p(s.cuda_stream))
    g.capture_end()
print(st)
"""


def test_first_transform_of_a_size_inside_capture_is_refused():
    """The first transform of a size builds its work grid and tables; inside
    a stream capture that is refused with LP_ERR_NOT_INITIALIZED."""
    import os
    import subprocess
    import sys
    from lightprop2d_gb300 import _lib as L
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "-c", _FIRST_TRANSFORM_IN_CAPTURE, root],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    assert int(p.stdout.strip().splitlines()[-1]) == L.LP_ERR_NOT_INITIALIZED
