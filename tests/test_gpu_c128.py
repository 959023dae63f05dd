"""GPU: the complex128 family (complex_bits=128, the reference's default
dtype) against numpy complex128 and the reference's own complex128 runs, to
round-off (relative L2 <= 1e-11).  The complex64 goldens of
test_gpu_beam2d.py run in both dtypes; this file adds the transforms, the
fused propagate with every multiplier, config 2 at 2048^2 and the argument
checks of the *_c128 entry points."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm = O.um, O.nm, O.mm
TOL128 = 1e-11


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))


@pytest.mark.parametrize("n", [2, 8, 16, 64, 75, 100, 512, 1024, 2048])
def test_fft2_c128(n):
    from lightprop2d_gb300 import backend as B
    x = _rand(n, n)
    t = torch.as_tensor(x, device="cuda")
    f = B.fft2(t)
    assert f.dtype == torch.complex128
    assert O.rel_l2(H(f), np.fft.fft2(x)) < TOL128
    assert O.rel_l2(H(B.ifft2(f)), x) < TOL128


@pytest.mark.parametrize("n", [4096, 8192])
def test_fft2_c128_large_plane_wave_and_round_trip(n):
    """4096 (in-place column pass with 1024-thread CTAs) and 8192 (transposes
    around a row pass): the transform of a plane wave is N^2 at its
    frequency and zero elsewhere, and ifft2(fft2(x)) returns x."""
    from lightprop2d_gb300 import backend as B
    a, b = 37, n - 5
    iy, ix = torch.meshgrid(torch.arange(n, dtype=torch.float64, device="cuda"),
                            torch.arange(n, dtype=torch.float64, device="cuda"), indexing="ij")
    x = torch.polar(torch.ones_like(iy), 2 * np.pi * ((a * iy + b * ix) % n) / n)
    f = B.fft2(x)
    peak = complex(f[a, b])
    assert abs(peak - n * n) < 1e-10 * n * n
    f[a, b] = 0
    assert float(torch.linalg.vector_norm(f)) < 1e-11 * n * n
    del f
    rng = np.random.default_rng(n)
    y = torch.as_tensor(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)), device="cuda")
    back = B.ifft2(B.fft2(y))
    assert float(torch.linalg.vector_norm(back - y) / torch.linalg.vector_norm(y)) < TOL128


@pytest.mark.parametrize("n,area,z", [(256, 0.05, 0.7), (100, 0.03, 0.2), (1024, 0.2, 3.0),
                                      (4096, 0.4, 2.0)])
def test_propagate_field_c128_with_every_multiplier(n, area, z):
    from lightprop2d_gb300 import backend as B
    wl = 632 * nm
    x = _rand(n, 2 * n)
    rng = np.random.default_rng(1)
    xm = rng.uniform(0.5, 1.0, size=(n, n))                      # float64 mask
    km = np.exp(2j * np.pi * rng.uniform(size=(n, n)))           # complex128 mask
    g = O.grids(area, n, wl)
    xr = x * O.lens_phase(g["X"], g["Y"], g["k0"], 7.0) * xm
    spec_z, want = O.propagate(O.fft2(xr) * km, g["Kz"], z)
    t = torch.as_tensor(x, device="cuda")
    s_out = torch.empty_like(t)
    ip = torch.empty((n, n), dtype=torch.float64, device="cuda")
    got = B.propagate_field(t, area, wl, z, spectrum_out=s_out, iprofile_out=ip, lens_f=7.0,
                            xmask=torch.as_tensor(xm, device="cuda"),
                            kmask=torch.as_tensor(km, device="cuda"))
    assert O.rel_l2(H(got), want) < TOL128
    assert O.rel_l2(H(s_out), spec_z) < TOL128
    assert np.linalg.norm(H(ip) - np.abs(want) ** 2) / np.linalg.norm(np.abs(want) ** 2) < TOL128


@pytest.mark.parametrize("n,area,z", [(256, 0.02, 0.9), (100, 0.01, 0.3), (2048, 0.2, 5.0)])
def test_propagate_c128_spectrum_state(n, area, z):
    """lp_propagate_c128 (Beam2D.propagate on the stored spectrum): H and a
    k-domain mask applied as the inverse transform loads the rows, the
    multiplied spectrum written back, against the oracle's complex128
    sequence (beam2d.py:481-490); also with the spectrum left unchanged."""
    from lightprop2d_gb300 import backend as B
    wl = 632 * nm
    x = _rand(n, 3 * n)
    g = O.grids(area, n, wl)
    km = np.exp(2j * np.pi * np.random.default_rng(2).uniform(size=(n, n)))
    spec = O.fft2(x)
    spec_z, want = O.propagate(spec * km, g["Kz"], z)
    t = torch.as_tensor(spec, device="cuda")
    f = B.propagate(t, area, wl, z, kmask=torch.as_tensor(km, device="cuda"))
    assert O.rel_l2(H(f), want) < TOL128
    assert O.rel_l2(H(t), spec_z) < TOL128
    t2 = torch.as_tensor(spec, device="cuda")
    _, want2 = O.propagate(spec, g["Kz"], z)
    f2 = B.propagate(t2, area, wl, z, write_spectrum=False)
    assert O.rel_l2(H(f2), want2) < TOL128
    assert np.array_equal(H(t2), spec)


@pytest.mark.parametrize("scale", [1e-20, 1e20])
def test_propagate_field_c128_far_from_unit_magnitude(scale):
    """The transforms carry float-float pairs (FP32's exponent range): fields
    far from unit magnitude keep complex128-level agreement."""
    from lightprop2d_gb300 import backend as B
    n, area, z, wl = 256, 0.05, 0.7, 632 * nm
    x = _rand(n, 7) * scale
    g = O.grids(area, n, wl)
    _, want = O.propagate(O.fft2(x), g["Kz"], z)
    got = B.propagate_field(torch.as_tensor(x, device="cuda"), area, wl, z)
    assert O.rel_l2(H(got), want) < TOL128


def test_config2_2048_c128_against_the_reference_run(golden):
    import lightprop2d_gb300 as lp
    b = lp.Beam2D(2 * mm, 2048, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 100 * um))      # complex_bits=128, the default
    assert b.field.dtype == torch.complex128
    for tag, dz in (("z1", 1.0), ("z10", 9.0)):
        b.propagate(dz)
        f = H(b.field)
        parts = {"window": f[992:1056, 992:1056], "row": f[1024, ::16], "col": f[::16, 1024]}
        for k, v in parts.items():
            assert O.rel_l2(v, golden[f"cfg2_{tag}_{k}"]) < 1e-10, (tag, k)
        e = float(np.sum(np.abs(f) ** 2))
        assert abs(e - float(golden[f"cfg2_{tag}_energy"])) < 1e-11 * e
    ip = b.iprofile
    assert ip.dtype == np.float64


def test_c128_argument_checks():
    from lightprop2d_gb300 import _lib as L
    lib = L.load()
    vp = ctypes.c_void_p
    x = torch.zeros((64, 64), dtype=torch.complex128, device="cuda")
    st = vp(torch.cuda.current_stream().cuda_stream)
    assert lib.lp_fft2_c128(vp(x.data_ptr()), vp(x.data_ptr()), 5000, 0, st) == \
        L.LP_ERR_UNSUPPORTED_SIZE
    assert lib.lp_fft2_c128(vp(x.data_ptr() + 8), vp(x.data_ptr()), 64, 0, st) == \
        L.LP_ERR_MISALIGNED
    assert lib.lp_propagate_field_c128(vp(x.data_ptr()), vp(x.data_ptr()), vp(0), vp(0), 64,
                                       0.1, 632e-7, 1.0, 0.0, vp(0), 0, vp(0), 0,
                                       L.LP_FLAG_ADJOINT, st) == L.LP_ERR_INVALID_ARGUMENT
