"""Pin the numpy oracle against golden vectors produced by the reference itself."""
import numpy as np
import pytest

from oracle import lp_oracle as O

um, nm, mm = O.um, O.nm, O.mm
TIGHT = 1e-12  # complex128 restatement vs complex128 reference


def test_cfg1_random_hole(golden):
    f0 = O.random_phase_hole(256, 200 * um, 25 * um, seed=int(golden["cfg1_seed"]))
    assert np.isclose(np.abs(f0).sum(), golden["cfg1_in_abs_sum"], rtol=0, atol=1e-9)
    b = O.OracleBeam(200 * um, 256, 632 * nm, init_field=f0)
    b.propagate(100 * um)
    assert O.rel_l2(b.field, golden["cfg1_field"]) < TIGHT
    assert np.allclose(b.iprofile.astype(np.float32), golden["cfg1_iprofile"], rtol=1e-6)


def test_sequential_propagate(golden):
    b = O.OracleBeam(2 * mm, 64, 632 * nm, init_field=golden["seq_in"])
    for i, dz in enumerate([0.1, 0.9, 4.0]):
        b.propagate(dz)
        assert O.rel_l2(b.field, golden[f"seq_field_{i}"]) < TIGHT
        assert O.rel_l2(b.spectrum, golden[f"seq_spectrum_{i}"]) < TIGHT
    assert b.z == golden["seq_z"]


def test_lens_then_propagate(golden):
    b = O.OracleBeam(500 * um, 64, 532 * nm, init_field=golden["lens_in"])
    b.lens(-0.1)
    assert O.rel_l2(b.field, golden["lens_field"]) < TIGHT
    assert O.rel_l2(b.spectrum, golden["lens_spectrum"]) < TIGHT
    b.propagate(0.02)
    assert O.rel_l2(b.field, golden["lens_prop_field"]) < TIGHT
    assert O.rel_l2(b.spectrum, golden["lens_prop_spectrum"]) < TIGHT


def test_filters(golden):
    b = O.OracleBeam(200 * um, 64, 632 * nm, init_field=golden["filt_in"])
    # round_hole generator, evaluated on the oracle grid (profiles.py:74-81)
    hole = np.exp(-(b.X ** 2 + b.Y ** 2) / (50 * um) ** 2) >= 1 / np.exp(0.5)
    b.coordinate_filter(hole)
    assert O.rel_l2(b.field, golden["filt_cf_gen_field"]) < TIGHT
    b.coordinate_filter(golden["filt_xmask"])
    assert O.rel_l2(b.field, golden["filt_cf_arr_field"]) < TIGHT
    assert O.rel_l2(b.spectrum, golden["filt_cf_arr_spectrum"]) < TIGHT
    b.spectral_filter(np.exp(-(b.Kx ** 2 + b.Ky ** 2) / 2000.0 ** 2))
    assert O.rel_l2(b.field, golden["filt_sf_gen_field"]) < TIGHT
    b.spectral_filter(golden["filt_kmask"])
    assert O.rel_l2(b.field, golden["filt_sf_arr_field"]) < TIGHT
    assert O.rel_l2(b.spectrum, golden["filt_sf_arr_spectrum"]) < TIGHT
    b.propagate(0.05)
    assert O.rel_l2(b.field, golden["filt_prop_field"]) < TIGHT


def test_evanescent_pass_through(golden):
    b = O.OracleBeam(20 * um, 64, 632 * nm, init_field=golden["evan_in"])
    assert np.mean(b.Kz == 0) == golden["evan_fraction"] > 0
    b.propagate(5 * um)
    assert O.rel_l2(b.field, golden["evan_field"]) < TIGHT


def test_negative_and_zero_z(golden):
    b = O.OracleBeam(1 * mm, 64, 1064 * nm, init_field=golden["negz_in"])
    b.propagate(0.3)
    assert O.rel_l2(b.field, golden["negz_fwd"]) < TIGHT
    b.propagate(0)
    assert O.rel_l2(b.field, golden["negz_zero"]) < TIGHT
    b.propagate(-0.3)
    assert O.rel_l2(b.field, golden["negz_back"]) < TIGHT
    assert b.z == golden["negz_z"]


def test_complex64_path(golden):
    f = O.gaussian(64, 2 * mm, 1, 100 * um)
    b = O.OracleBeam(2 * mm, 64, 632 * nm, init_field=f, complex_bits=64)
    b.propagate(1.0)
    assert b.field.dtype == np.complex64
    assert O.rel_l2(b.field, golden["c64_field"]) < 1e-6


def test_init_spectrum_is_state(golden):
    b = O.OracleBeam(300 * um, 64, 800 * nm, init_field=golden["ispec_field_in"],
                     init_spectrum=golden["ispec_spectrum_in"])
    b.propagate(0.01)
    assert O.rel_l2(b.field, golden["ispec_field"]) < TIGHT


def test_mixed_sequence(golden):
    b = O.OracleBeam(400 * um, 64, 700 * nm, init_field=golden["mix_in"])
    b.lens(2.0)
    b.propagate(0.5)
    sq = (np.abs(b.X) < 75 * um) & (np.abs(b.Y) < 75 * um)
    b.coordinate_filter(sq)
    b.propagate(0.25)
    b.spectral_filter(golden["filt_kmask"])
    b.propagate(-0.1)
    assert O.rel_l2(b.field, golden["mix_field"]) < TIGHT
    assert O.rel_l2(b.spectrum, golden["mix_spectrum"]) < TIGHT
    assert np.isclose(b.z, golden["mix_z"])


def test_config2_oracle_vs_analytic_gaussian():
    """2048^2, 2 mm, 632 nm, waist 100 um: the oracle's angular spectrum
    against the analytic paraxial Gaussian at z = 0.1..10 cm (the departure
    grows linearly with z: non-paraxial terms)."""
    n, area, wl, w0 = 2048, 2 * mm, 632 * nm, 100 * um
    g = O.grids(area, n, wl)
    s0 = np.fft.fft2(O.gaussian(n, area, 1.0, w0))
    for z in (0.1, 1.0, 5.0, 10.0):
        _, f = O.propagate(s0, g["Kz"], z)
        e = O.rel_l2(f, O.gaussian_paraxial(n, area, wl, w0, z))
        assert e < 3e-7 * z, (z, e)


@pytest.mark.parametrize("tag", ["a8", "a16"])
def test_gaussian_known_answer(golden, tag):
    """On-axis intensity vs 1/(1+z_n^2) (tests/test_analytics.py:53-71)."""
    R, k0 = float(golden[f"kat_{tag}_R"]), float(golden[f"kat_{tag}_k0"])
    zs = np.arange(20) * 0.02
    theory = 1 / (1 + (zs / 2 / np.pi / k0 / R ** 2) ** 2)
    assert np.allclose(golden[f"kat_{tag}_I"], theory, rtol=1e-2)
    b = O.OracleBeam(3 * mm, 512, 632 * nm, init_field=O.gaussian(512, 3 * mm, 1, R))
    b.propagate(zs[0])
    vals = []
    for _ in zs:
        vals.append(b.iprofile[256, 256])
        b.propagate(0.02)
    assert np.allclose(vals, golden[f"kat_{tag}_I"], rtol=1e-12)


def test_metrics_and_grid_oracle_match_reference(golden):
    """Oracle restatements of centroid / D4sigma / centroid_intensity
    (beam2d.py:669-752), expand and coarse (beam2d.py:375-460) reproduce the
    reference's own outputs; crop's interp2d (gone from SciPy >= 1.14, the
    reference raises there) is checked against SciPy's linear
    RegularGridInterpolator with nearest-value clamping."""
    b = golden["cfg1_field"]
    dL = O.um * 200 / 256
    m = [*O.centroid(b, dL), *O.d4sigma(b, dL), O.centroid_intensity(b, dL)]
    assert np.allclose(m, golden["met_cfg1"], rtol=1e-12, atol=0)
    assert np.array_equal(O.expand(golden["grid_in"], int(golden["grid_expand_n"])),
                          golden["grid_expand_field"])
    c = O.coarse(golden["grid_expand_field"], 2)
    assert np.allclose(c, golden["grid_coarse_field"], rtol=1e-6, atol=1e-7)
    assert not bool(golden["grid_crop_runs"])
    from scipy.interpolate import RegularGridInterpolator
    X = np.arange(-64, 64) * (0.1 / 128)
    f = golden["grid_in"]
    keep = X[np.abs(X) < 0.025]
    nc, n = 64, len(keep) // 2
    ox, win = X[nc - n:nc + n], f[nc - n:nc + n, nc - n:nc + n]
    qx = np.arange(-40, 40) * (0.06 / 80)
    q = np.clip(qx, ox[0], ox[-1])
    ref = RegularGridInterpolator((ox, ox), win)(np.stack(np.meshgrid(q, q, indexing="ij"), -1))
    assert np.allclose(O.crop(f, X, 0.05, 80, 0.06), ref, rtol=1e-12, atol=1e-15)


def test_modes_oracle_matches_reference(golden):
    f, m = golden["modes_field"], golden["modes_basis"]
    assert np.allclose(O.modes_scalar(f, m), golden["modes_scalar"], rtol=1e-12, atol=0)
    assert np.allclose(O.modes_lstsq(f, m), golden["modes_lstsq"], rtol=1e-9, atol=1e-12)
    mt = np.vstack(m).T
    assert np.allclose(O.modes_fast(f, mt.T, mt.T.dot(mt)), golden["modes_fast"], rtol=1e-9)
    c = golden["modes_scalar"] * np.exp(0.5j)
    assert np.allclose(O.modes_combine(m, c, 64), golden["modes_constructed"], rtol=1e-12,
                       atol=1e-15)


def _cfg2_parts(f, tag):
    return {"window": f[992:1056, 992:1056], "row": f[1024, ::16], "col": f[::16, 1024]}


def test_config2_2048_reference_run(golden):
    """Config 2 at its full size (2048^2): the oracle against the reference's
    own complex128 run at z = 1 cm and 10 cm (window, centre row/column,
    energy)."""
    b = O.OracleBeam(2 * mm, 2048, 632 * nm, init_field=O.gaussian(2048, 2 * mm, 1, 100 * um))
    for tag, dz in (("z1", 1.0), ("z10", 9.0)):
        b.propagate(dz)
        for k, v in _cfg2_parts(b.field, tag).items():
            assert O.rel_l2(v, golden[f"cfg2_{tag}_{k}"]) < 1e-10, (tag, k)
        e = np.sum(np.abs(b.field) ** 2)
        assert abs(e - golden[f"cfg2_{tag}_energy"]) < 1e-10 * e


@pytest.mark.parametrize("n,tag", [(100, "np100"), (75, "np75")])
def test_sizes_not_powers_of_two(golden, n, tag):
    """Even and odd npoints that are not powers of two: lens, propagate,
    round-hole and Gaussian filters, against the reference's own run."""
    b = O.OracleBeam(1 * mm, n, 632 * nm, init_field=golden[f"{tag}_in"])
    b.lens(5.0)
    b.propagate(0.3)
    assert O.rel_l2(b.field, golden[f"{tag}_lens_prop_field"]) < TIGHT
    assert O.rel_l2(b.spectrum, golden[f"{tag}_lens_prop_spectrum"]) < TIGHT
    hole = np.exp(-(b.X ** 2 + b.Y ** 2) / (300 * um) ** 2) >= 1 / np.exp(0.5)
    b.coordinate_filter(hole)
    b.spectral_filter(np.exp(-(b.Kx ** 2 + b.Ky ** 2) / 2e4 ** 2))
    b.propagate(0.5)
    assert O.rel_l2(b.field, golden[f"{tag}_filt_prop_field"]) < TIGHT
    assert np.allclose(b.iprofile, golden[f"{tag}_filt_prop_iprofile"], rtol=1e-10, atol=1e-14)
