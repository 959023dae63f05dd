"""GPU parity: CUDA kernels (through the C ABI) vs the numpy oracle.

Tolerance: relative L2 <= 1e-5 against the complex128 oracle for every field
result (the bar of the reference's complex64 path is ~1.5e-7); energy error
<= 1e-5.  FFT-only checks use 2e-6.
"""
import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm = O.um, O.nm, O.mm
TOL = 1e-5
FFT_TOL = 2e-6
SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096]


@pytest.fixture(scope="module")
def B():
    from lightprop2d_gb300 import backend
    backend.init(0)
    return backend


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda").to(torch.complex64)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rand_field(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))


@pytest.mark.parametrize("n", SIZES)
def test_fft2_ifft2(B, n):
    x = rand_field(n, n)
    X = B.fft2(dev(x))
    assert O.rel_l2(host(X), np.fft.fft2(x)) < FFT_TOL
    y = B.ifft2(dev(x))
    assert O.rel_l2(host(y), np.fft.ifft2(x)) < FFT_TOL
    # in place
    t = dev(x)
    B.fft2(t, out=t)
    assert O.rel_l2(host(t), np.fft.fft2(x)) < FFT_TOL


@pytest.mark.parametrize("n", SIZES)
def test_propagate_spectrum_state(B, n):
    """lp_propagate: spectrum *= H, field = ifft2(spectrum) (beam2d.py:484-490)."""
    area, wl, z = 2 * mm * n / 2048 * 4, 632 * nm, 0.37
    g = O.grids(area, n, wl)
    s = np.fft.fft2(rand_field(n, 3 + n))
    s_ref, f_ref = O.propagate(s, g["Kz"], z)
    st = dev(s)
    f = B.propagate(st, area, wl, z)
    assert O.rel_l2(host(f), f_ref) < TOL
    assert O.rel_l2(host(st), s_ref) < TOL
    assert O.energy_err(host(f), f_ref) < TOL


@pytest.mark.parametrize("n", SIZES)
def test_propagate_field_fused(B, n):
    """Fused lens + mask + propagate + iprofile vs the oracle sequence."""
    area, wl, z, f = 1 * mm, 1064 * nm, 0.8, 3.0
    g = O.grids(area, n, wl)
    rng = np.random.default_rng(n)
    x = rand_field(n, 7 * n)
    xm = rng.uniform(0.2, 1.0, size=(n, n)).astype(np.float32)
    km = (rng.uniform(0.5, 1, (n, n)) * np.exp(1j * rng.uniform(0, 6.28, (n, n)))).astype(np.complex64)
    fl, _ = O.lens(x, g["X"], g["Y"], g["k0"], f)
    fl, _ = O.coordinate_filter(fl, xm.astype(np.float64))
    s = np.fft.fft2(fl) * km.astype(np.complex128)
    s_ref, f_ref = O.propagate(s, g["Kz"], z)
    spec = torch.empty((n, n), dtype=torch.complex64, device="cuda")
    ip = torch.empty((n, n), dtype=torch.float32, device="cuda")
    out = B.propagate_field(dev(x), area, wl, z, spectrum_out=spec, iprofile_out=ip,
                            lens_f=f, xmask=torch.as_tensor(xm, device="cuda"),
                            kmask=torch.as_tensor(km, device="cuda"))
    assert O.rel_l2(host(out), f_ref) < TOL
    assert O.rel_l2(host(spec), s_ref) < TOL
    assert np.allclose(host(ip), np.abs(f_ref) ** 2, rtol=1e-4, atol=1e-6 * np.abs(f_ref).max() ** 2)


@pytest.mark.parametrize("n,area,wl,z", [
    (2048, 0.10409037570395337, 1064 * nm, 1.7394964232143395),
    (2048, 0.04663, 632 * nm, 1.87),
    (1024, 0.05, 1064 * nm, 3.3),
    (1024, 0.025, 532 * nm, 12.0),
    (4096, 0.1, 632 * nm, 5.0),
    (512, 0.012, 632 * nm, 3.7)])
def test_near_evanescent_cutoff(B, n, area, wl, z):
    """White-spectrum fields on grids finer than wl/2 put energy at the
    evanescent cut-off, where kz*z = R*sqrt(v) with v -> 0 after cancellation;
    the float-float phase must stay within the bar there too."""
    g = O.grids(area, n, wl)
    assert area / n < wl / 2
    x = O.random_phase_hole(n, area, 0.3 * area, seed=n + 1)
    _, f_ref = O.propagate(np.fft.fft2(x), g["Kz"], z)
    out = B.propagate_field(dev(x), area, wl, z)
    assert O.rel_l2(host(out), f_ref) < TOL
    s = B.propagate(dev(np.fft.fft2(x)), area, wl, z, write_spectrum=False)
    assert O.rel_l2(host(s), f_ref) < TOL


def test_config2_gaussian_2048_all_z(B):
    """2048^2, 2 mm, 632 nm, waist 100 um, z in {0.1,1,5,10,50} cm.

    Float-float phase (the product path) meets 1e-5 at every z; the plain-FP32
    phase variant degrades with z (reported side by side in bench)."""
    n, area, wl = 2048, 2 * mm, 632 * nm
    g = O.grids(area, n, wl)
    f0 = O.gaussian(n, area, 1, 100 * um)
    s0 = np.fft.fft2(f0)
    from lightprop2d_gb300 import _lib as L
    errs_ff, errs_32 = [], []
    for z in (0.1, 1, 5, 10, 50):
        _, f_ref = O.propagate(s0, g["Kz"], z)
        f = B.propagate(dev(s0), area, wl, z, write_spectrum=False)
        errs_ff.append(O.rel_l2(host(f), f_ref))
        f32 = B.propagate(dev(s0), area, wl, z, write_spectrum=False, flags=L.LP_FLAG_PHASE_FP32)
        errs_32.append(O.rel_l2(host(f32), f_ref))
        ff = B.propagate_field(dev(f0), area, wl, z)
        assert O.rel_l2(host(ff), f_ref) < TOL
    assert max(errs_ff) < TOL, errs_ff
    assert errs_32[-1] > 10 * errs_ff[-1], (errs_32, errs_ff)


def test_config2_vs_analytic_gaussian(B):
    """The fused GPU propagate of config 2 against the analytic paraxial
    Gaussian (z <= 10 cm; at 50 cm the beam wraps in the window): the
    departure is the oracle's own non-paraxial term plus FP32 round-off."""
    n, area, wl, w0 = 2048, 2 * mm, 632 * nm, 100 * um
    f0 = O.gaussian(n, area, 1.0, w0)
    for z in (0.1, 1.0, 5.0, 10.0):
        f = host(B.propagate_field(dev(f0), area, wl, z))
        e = O.rel_l2(f, O.gaussian_paraxial(n, area, wl, w0, z))
        assert e < 3e-7 * z + 1e-6, (z, e)


def test_plain_matches_fused(B):
    n, area, wl, z = 1024, 2 * mm, 632 * nm, 2.5
    g = O.grids(area, n, wl)
    x = rand_field(n, 5)
    _, f_ref = O.propagate(np.fft.fft2(x), g["Kz"], z)
    p = B.plain_propagate_field(dev(x), area, wl, z)
    p64 = B.plain_propagate_field(dev(x), area, wl, z, fp64_h=True)
    fu = B.propagate_field(dev(x), area, wl, z)
    assert O.rel_l2(host(p), f_ref) < TOL
    assert O.rel_l2(host(p64), f_ref) < TOL
    assert O.rel_l2(host(fu), f_ref) < TOL


@pytest.mark.parametrize("n", [256, 2048, 4096])
def test_phase_mask_large_phases(B, n):
    """An FP32 phase mask far outside [-pi, pi] (|phi| up to 800 rad) in the
    first pass (register and TMA row kernels) and, with XMASK_AFTER, on the
    store side of the last pass, against exp(1j*phi) in float64."""
    from lightprop2d_gb300 import _lib as L
    area, wl, z = 1 * mm, 632 * nm, 0.5
    rng = np.random.default_rng(n + 5)
    x = O.random_phase_hole(n, area, 0.3 * area, seed=n + 7)
    phi = rng.uniform(-800.0, 800.0, (n, n)).astype(np.float32)
    pm = torch.as_tensor(phi, device="cuda")
    mult = np.exp(1j * phi.astype(np.float64))
    g = O.grids(area, n, wl)
    _, ref = O.propagate(np.fft.fft2(x * mult), g["Kz"], z)
    got = host(B.propagate_field(dev(x), area, wl, z, xmask=pm, xmask_phase=True))
    assert O.rel_l2(got, ref) < TOL
    _, ref2 = O.propagate(np.fft.fft2(x), g["Kz"], z)
    got2 = host(B.propagate_field(dev(x), area, wl, z, xmask=pm, xmask_phase=True,
                                  flags=L.LP_FLAG_XMASK_AFTER))
    assert O.rel_l2(got2, ref2 * mult) < TOL


def test_adjoint_identity(B):
    """<P u, v> == <u, P^H v> for the fused operator with lens and masks."""
    from lightprop2d_gb300 import _lib as L
    n, area, wl, z, f = 256, 500 * um, 800 * nm, 0.3, 1.5
    rng = np.random.default_rng(2)
    u, v = rand_field(n, 11), rand_field(n, 12)
    xm = torch.as_tensor(rng.uniform(0, 6.28, (n, n)).astype(np.float32), device="cuda")
    km = torch.as_tensor(rng.uniform(0.3, 1, (n, n)).astype(np.float32), device="cuda")
    Pu = host(B.propagate_field(dev(u), area, wl, z, lens_f=f, xmask=xm, xmask_phase=True,
                                kmask=km))
    PHv = host(B.propagate_field(dev(v), area, wl, z, lens_f=f, xmask=xm, xmask_phase=True,
                                 kmask=km, flags=L.LP_FLAG_ADJOINT))
    lhs = np.vdot(v, Pu)
    rhs = np.vdot(PHv, u)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_dz_derivative(B):
    """LP_FLAG_DZ gives d/dz of the propagated field (central difference in
    complex128; the step keeps the carrier phase change 2*pi*k0*h ~ 1e-3 rad)."""
    from lightprop2d_gb300 import _lib as L
    n, area, wl, z, h = 256, 1 * mm, 632 * nm, 0.5, 1e-8
    x = O.gaussian(n, area, 1, 80 * um) * np.exp(1j * 0.3)
    d = host(B.propagate_field(dev(x), area, wl, z, flags=L.LP_FLAG_DZ))
    g = O.grids(area, n, wl)
    fp = O.propagate(np.fft.fft2(x), g["Kz"], z + h)[1]
    fm = O.propagate(np.fft.fft2(x), g["Kz"], z - h)[1]
    fd = (fp - fm) / (2 * h)
    assert O.rel_l2(d, fd) < 1e-3


def test_evanescent_mask_flag(B):
    from lightprop2d_gb300 import _lib as L
    n, area, wl, z = 64, 20 * um, 632 * nm, 5 * um
    g = O.grids(area, n, wl)
    x = rand_field(n, 9)
    s = np.fft.fft2(x)
    H = O.transfer(g["Kz"], z)
    H[g["Kz"] == 0] = 0
    ref = np.fft.ifft2(s * H)
    f = B.propagate(dev(s), area, wl, z, write_spectrum=False, flags=L.LP_FLAG_EVANESCENT_MASK)
    assert O.rel_l2(host(f), ref) < TOL


def test_iprofile_and_apply_transfer(B):
    n, area, wl, z = 512, 1 * mm, 532 * nm, 1.3
    x = rand_field(n, 4)
    ip = host(B.iprofile(dev(x)))
    assert np.allclose(ip, np.abs(x.astype(np.complex64)) ** 2, rtol=1e-6)
    g = O.grids(area, n, wl)
    s = dev(x)
    B.apply_transfer(s, area, wl, z)
    assert O.rel_l2(host(s), x * O.transfer(g["Kz"], z)) < TOL


@pytest.mark.parametrize("n", [1024, 2048, 4096])
def test_tma_and_register_row_paths_agree(B, n):
    """At 4096, 16-byte aligned grids take the TMA-staged row kernels and a
    grid that is only 8-byte aligned takes the register-prefetch kernels
    (which every grid of 1024-2048 uses).  All match the oracle, in place and
    out of place, and no bounded wait gave up."""
    from lightprop2d_gb300 import _lib as L
    area, wl, z, f = 1 * mm, 632 * nm, 2.0, 4.0
    g = O.grids(area, n, wl)
    x = rand_field(n, 3 * n)
    fl, _ = O.lens(x, g["X"], g["Y"], g["k0"], f)
    _, f_ref = O.propagate(np.fft.fft2(fl), g["Kz"], z)
    a = dev(x)
    assert a.data_ptr() % 16 == 0
    raw = torch.empty(n * n + 1, dtype=torch.complex64, device="cuda")
    b = raw[1:].view(n, n)
    assert b.data_ptr() % 16 == 8
    b.copy_(a)
    ip = torch.empty((n, n), dtype=torch.float32, device="cuda")
    out_a = B.propagate_field(a, area, wl, z, lens_f=f, iprofile_out=ip)
    out_b = B.propagate_field(b, area, wl, z, lens_f=f)
    assert O.rel_l2(host(out_a), f_ref) < TOL
    assert O.rel_l2(host(out_b), f_ref) < TOL
    assert np.allclose(host(ip), np.abs(host(out_a)) ** 2, rtol=1e-5, atol=1e-7)
    B.propagate_field(a, area, wl, z, out=a, lens_f=f)      # in place
    assert O.rel_l2(host(a), f_ref) < TOL
    s = B.fft2(dev(x))
    assert O.rel_l2(host(s), np.fft.fft2(x)) < FFT_TOL
    st = torch.cuda.current_stream()
    L.check(L.load().lp_async_status(ctypes_vp(st.cuda_stream)), "lp_async_status")


def ctypes_vp(v):
    import ctypes
    return ctypes.c_void_p(v)


def test_errors_are_raised(B):
    with pytest.raises(ValueError):
        B.fft2(torch.zeros((1, 1), dtype=torch.complex64, device="cuda"))  # npoints 1
    with pytest.raises(ValueError):
        B.fft2(torch.zeros((64, 64), dtype=torch.float32, device="cuda"))  # not complex
    with pytest.raises(ValueError):
        B.propagate(torch.zeros((64, 64), dtype=torch.complex64, device="cuda"), -1.0, 1e-4, 1.0)


@pytest.mark.parametrize("n", [256, 1024, 2048, 4096])
def test_specialised_and_general_kernels_agree(B, n):
    """The launcher runs kernels compiled for what a call uses: transform-only
    row passes and an H-only column pass when there is no multiplier, an
    FP32-phase-mask row pass for a phase mask alone.  Adding a multiplier of
    value one (an all-ones k mask, an iprofile epilogue) sends the same call
    through the general kernels; both must match the oracle and each other."""
    from lightprop2d_gb300 import _lib as L
    area, wl, z = 1 * mm, 632 * nm, 1.3
    g = O.grids(area, n, wl)
    x = rand_field(n, 5 * n + 1)
    _, f_ref = O.propagate(np.fft.fft2(x), g["Kz"], z)
    ones = torch.ones((n, n), dtype=torch.float32, device="cuda")
    lean = host(B.propagate_field(dev(x), area, wl, z))
    ip = torch.empty((n, n), dtype=torch.float32, device="cuda")
    general = host(B.propagate_field(dev(x), area, wl, z, kmask=ones, iprofile_out=ip))
    assert O.rel_l2(lean, f_ref) < TOL
    assert O.rel_l2(general, f_ref) < TOL
    assert O.rel_l2(lean, general) < 1e-6
    # FP32 phase mask alone (before and after the transform) vs with an epilogue
    rng = np.random.default_rng(n)
    phi = rng.uniform(-20.0, 20.0, (n, n)).astype(np.float32)
    pm = torch.as_tensor(phi, device="cuda")
    mult = np.exp(1j * phi.astype(np.float64))
    _, ref_before = O.propagate(np.fft.fft2(x * mult), g["Kz"], z)
    cm = torch.as_tensor(mult.astype(np.complex64), device="cuda")
    # before the transform: the phase-mask row kernel vs a complex64 mask of
    # the same values (general kernel); after it: alone vs with an epilogue
    a = host(B.propagate_field(dev(x), area, wl, z, xmask=pm, xmask_phase=True))
    b = host(B.propagate_field(dev(x), area, wl, z, xmask=cm))
    assert O.rel_l2(a, ref_before) < TOL
    assert O.rel_l2(b, ref_before) < TOL
    assert O.rel_l2(a, b) < 2e-6
    after = L.LP_FLAG_XMASK_AFTER
    a = host(B.propagate_field(dev(x), area, wl, z, xmask=pm, xmask_phase=True, flags=after))
    b = host(B.propagate_field(dev(x), area, wl, z, xmask=pm, xmask_phase=True, flags=after,
                               iprofile_out=ip))
    assert O.rel_l2(a, f_ref * mult) < TOL
    assert O.rel_l2(b, f_ref * mult) < TOL
    assert O.rel_l2(a, b) < 1e-6
