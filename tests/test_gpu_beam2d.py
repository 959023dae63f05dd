"""GPU: the Beam2D drop-in reproduces the reference's own outputs (golden vectors)."""
import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm = O.um, O.nm, O.mm
TOL = 1e-5
# complex_bits=128 (the reference's default) runs the FP64 kernel family: it
# must reproduce the reference's complex128 outputs to round-off.
TOL128 = 1e-11


@pytest.fixture(params=[64, 128])
def bits(request):
    return request.param


def tol(bits):
    return TOL if bits == 64 else TOL128


@pytest.fixture(scope="module")
def lp():
    import lightprop2d_gb300 as lp
    return lp


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy() if isinstance(t, torch.Tensor) else t


def test_cfg1_random_hole_256(lp, golden, bits):
    f0 = O.random_phase_hole(256, 200 * um, 25 * um, seed=int(golden["cfg1_seed"]))
    b = lp.Beam2D(200 * um, 256, 632 * nm, init_field=f0, complex_bits=bits)
    b.propagate(100 * um)
    assert O.rel_l2(H(b.field), golden["cfg1_field"]) < tol(bits)
    ip = b.iprofile
    assert isinstance(ip, np.ndarray)
    assert ip.dtype == (np.float32 if bits == 64 else np.float64)  # the reference's dtypes
    ref = golden["cfg1_iprofile"].astype(np.float64)  # stored as float32
    assert np.linalg.norm(ip - ref) / np.linalg.norm(ref) < 2 * TOL


def test_sequential(lp, golden, bits):
    b = lp.Beam2D(2 * mm, 64, 632 * nm, init_field=golden["seq_in"], complex_bits=bits)
    for i, dz in enumerate([0.1, 0.9, 4.0]):
        b.propagate(dz)
        assert O.rel_l2(H(b.field), golden[f"seq_field_{i}"]) < tol(bits)
        assert O.rel_l2(H(b.spectrum), golden[f"seq_spectrum_{i}"]) < tol(bits)
    assert b.z == golden["seq_z"]


def test_lens(lp, golden, bits):
    b = lp.Beam2D(500 * um, 64, 532 * nm, init_field=golden["lens_in"], complex_bits=bits)
    b.lens(-0.1)
    assert O.rel_l2(H(b.field), golden["lens_field"]) < tol(bits)
    assert O.rel_l2(H(b.spectrum), golden["lens_spectrum"]) < tol(bits)
    b.propagate(0.02)
    assert O.rel_l2(H(b.field), golden["lens_prop_field"]) < tol(bits)
    assert O.rel_l2(H(b.spectrum), golden["lens_prop_spectrum"]) < tol(bits)


def test_lens_fused_without_intermediate_read(lp, golden, bits):
    b = lp.Beam2D(500 * um, 64, 532 * nm, init_field=golden["lens_in"], complex_bits=bits)
    b.lens(-0.1)
    b.propagate(0.02)   # lens folded into the fused pass sequence
    assert O.rel_l2(H(b.field), golden["lens_prop_field"]) < tol(bits)
    assert O.rel_l2(H(b.spectrum), golden["lens_prop_spectrum"]) < tol(bits)


def test_filters(lp, golden, bits):
    b = lp.Beam2D(200 * um, 64, 632 * nm, init_field=golden["filt_in"], complex_bits=bits)
    b.coordinate_filter(f_gen=lp.round_hole, fargs=(50 * um,))
    assert O.rel_l2(H(b.field), golden["filt_cf_gen_field"]) < tol(bits)
    b.coordinate_filter(f_init=golden["filt_xmask"])
    assert O.rel_l2(H(b.field), golden["filt_cf_arr_field"]) < tol(bits)
    assert O.rel_l2(H(b.spectrum), golden["filt_cf_arr_spectrum"]) < tol(bits)
    b.spectral_filter(f_gen=lambda kx, ky, s: np.exp(-(kx ** 2 + ky ** 2) / s ** 2),
                      fargs=(2000.0,))
    assert O.rel_l2(H(b.field), golden["filt_sf_gen_field"]) < tol(bits)
    b.spectral_filter(f_init=golden["filt_kmask"])
    assert O.rel_l2(H(b.field), golden["filt_sf_arr_field"]) < tol(bits)
    assert O.rel_l2(H(b.spectrum), golden["filt_sf_arr_spectrum"]) < tol(bits)
    b.propagate(0.05)
    assert O.rel_l2(H(b.field), golden["filt_prop_field"]) < tol(bits)


def test_evanescent(lp, golden, bits):
    b = lp.Beam2D(20 * um, 64, 632 * nm, init_field=golden["evan_in"], complex_bits=bits)
    assert np.mean(b.Kz == 0) == golden["evan_fraction"]
    b.propagate(5 * um)
    assert O.rel_l2(H(b.field), golden["evan_field"]) < tol(bits)


def test_negative_and_zero_z(lp, golden, bits):
    b = lp.Beam2D(1 * mm, 64, 1064 * nm, init_field=golden["negz_in"], complex_bits=bits)
    b.propagate(0.3)
    assert O.rel_l2(H(b.field), golden["negz_fwd"]) < tol(bits)
    b.propagate(0)
    assert O.rel_l2(H(b.field), golden["negz_zero"]) < tol(bits)
    b.propagate(-0.3)
    assert O.rel_l2(H(b.field), golden["negz_back"]) < tol(bits)
    assert b.z == golden["negz_z"]


def test_complex64_request(lp, golden):
    b = lp.Beam2D(2 * mm, 64, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 100 * um), complex_bits=64)
    b.propagate(1.0)
    assert b.field.dtype == torch.complex64
    assert O.rel_l2(H(b.field), golden["c64_field"]) < TOL


def test_init_spectrum_is_state(lp, golden, bits):
    b = lp.Beam2D(300 * um, 64, 800 * nm, init_field=golden["ispec_field_in"],
                  init_spectrum=golden["ispec_spectrum_in"], complex_bits=bits)
    b.propagate(0.01)
    assert O.rel_l2(H(b.field), golden["ispec_field"]) < tol(bits)


def test_mixed_sequence(lp, golden, bits):
    b = lp.Beam2D(400 * um, 64, 700 * nm, init_field=golden["mix_in"], complex_bits=bits)
    b.lens(2.0)
    b.propagate(0.5)
    b.coordinate_filter(f_gen=lp.square_hole, fargs=(150 * um,))
    b.propagate(0.25)
    b.spectral_filter(f_init=golden["filt_kmask"])
    b.propagate(-0.1)
    assert O.rel_l2(H(b.field), golden["mix_field"]) < tol(bits)
    assert O.rel_l2(H(b.spectrum), golden["mix_spectrum"]) < tol(bits)
    assert np.isclose(b.z, golden["mix_z"])


@pytest.mark.parametrize("tag", ["a8", "a16"])
def test_gaussian_known_answer_512(lp, golden, tag):
    """tests/test_analytics.py:53-71: on-axis intensity vs the reference run."""
    R = float(golden[f"kat_{tag}_R"])
    b = lp.Beam2D(3 * mm, 512, 632 * nm, init_field_gen=lp.gaussian_beam, init_gen_args=(1, R))
    zs = np.arange(20) * 0.02
    b.propagate(zs[0])
    vals = []
    for _ in zs:
        vals.append(b.iprofile[256, 256])
        b.propagate(0.02)
    assert np.allclose(vals, golden[f"kat_{tag}_I"], rtol=1e-5)
    theory = 1 / (1 + (zs / 2 / np.pi / b.k0 / R ** 2) ** 2)
    assert np.allclose(vals, theory, rtol=1e-2)


def test_field_assignment_keeps_spectrum(lp):
    """Direct field assignment leaves the spectrum (reference dataclass semantics)."""
    f0 = O.gaussian(64, 1 * mm, 1, 100 * um)
    b = lp.Beam2D(1 * mm, 64, 632 * nm, init_field=f0)
    s_before = H(b.spectrum).copy()
    b.field = np.zeros((64, 64), np.complex64)
    assert O.rel_l2(H(b.spectrum), s_before) == 0
    b.propagate(0.1)  # propagates the stored spectrum, not the zero field
    g = O.grids(1 * mm, 64, 632 * nm)
    assert O.rel_l2(H(b.field), O.propagate(np.fft.fft2(f0), g["Kz"], 0.1)[1]) < TOL


def test_unsupported_npoints(lp):
    with pytest.raises(ValueError):
        lp.Beam2D(1 * mm, 5000, 632 * nm, init_field=np.ones((1, 1)))


def test_missing_init_raises(lp):
    with pytest.raises(ValueError):
        lp.Beam2D(1 * mm, 64, 632 * nm)


def test_config2_2048_against_the_reference_run(lp, golden):
    """Config 2 (Gaussian 2048^2, area 2 mm, 632 nm, waist 100 um) through
    Beam2D in complex64 against the reference's own complex128 run at
    z = 1 cm and 10 cm: central window, centre row and column, energy."""
    b = lp.Beam2D(2 * mm, 2048, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 100 * um), complex_bits=64)
    for tag, dz in (("z1", 1.0), ("z10", 9.0)):
        b.propagate(dz)
        f = H(b.field)
        parts = {"window": f[992:1056, 992:1056], "row": f[1024, ::16], "col": f[::16, 1024]}
        for k, v in parts.items():
            assert O.rel_l2(v, golden[f"cfg2_{tag}_{k}"]) < TOL, (tag, k)
        e = float(np.sum(np.abs(f.astype(np.complex128)) ** 2))
        assert abs(e - float(golden[f"cfg2_{tag}_energy"])) < TOL * e
