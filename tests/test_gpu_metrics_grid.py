"""GPU: beam metrics (lp_beam_moments) and grid management (lp_expand,
lp_coarse, lp_crop, lens_image) against the reference's own outputs (golden
vectors) and the oracle."""
import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm = O.um, O.nm, O.mm


@pytest.fixture(scope="module")
def lp():
    import lightprop2d_gb300 as lp
    return lp


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy() if isinstance(t, torch.Tensor) else t


def metrics(b):
    Xc, Yc, nxc, nyc = b.centroid
    dx, dy = b.D4sigma
    return np.array([Xc, Yc, nxc, nyc, dx, dy, b.centroid_intensity])


def check_metrics(got, ref, dL):
    assert abs(got[0] - ref[0]) < 1e-5 * dL and abs(got[1] - ref[1]) < 1e-5 * dL, (got, ref)
    assert got[2] == ref[2] and got[3] == ref[3]
    assert np.allclose(got[4:6], ref[4:6], rtol=1e-5)
    assert np.isclose(got[6], ref[6], rtol=2e-5)


def test_metrics_match_reference(lp, golden):
    f0 = O.random_phase_hole(256, 200 * um, 25 * um, seed=int(golden["cfg1_seed"]))
    b = lp.Beam2D(200 * um, 256, 632 * nm, init_field=f0)
    b.propagate(100 * um)
    check_metrics(metrics(b), golden["met_cfg1"], b.dL)
    M = lp.Beam2D(1 * mm, 512, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 50 * um, 200 * um, -150 * um), complex_bits=64)
    check_metrics(metrics(M), golden["met_off_in"], M.dL)
    M.lens(3.0)
    M.propagate(2.0)
    check_metrics(metrics(M), golden["met_off_prop"], M.dL)


@pytest.mark.parametrize("n", [16, 64, 1024, 2048, 4096])
def test_metrics_vs_oracle_off_centre(lp, n):
    area = 2 * mm
    g = O.grids(area, n, 632 * nm)
    x = O.gaussian(n, area, 1.0, area / 12) * np.exp(1j * 0.3)
    x = np.roll(x, (n // 5, -n // 7), axis=(0, 1))       # far off centre
    x = x + 0.05 * O.random_phase_hole(n, area, area / 3, seed=n)
    b = lp.Beam2D(area, n, 632 * nm, init_field=x)
    xf = H(b.field).astype(np.complex128)
    ref = np.array([*O.centroid(xf, g["dL"]), *O.d4sigma(xf, g["dL"]),
                    O.centroid_intensity(xf, g["dL"])])
    check_metrics(metrics(b), ref, g["dL"])


def test_metrics_zero_field(lp):
    b = lp.Beam2D(1 * mm, 64, 632 * nm, init_field=np.zeros((64, 64)))
    with pytest.raises(ZeroDivisionError):
        b.centroid


def test_expand_coarse_match_reference(lp, golden):
    G = lp.Beam2D(1 * mm, 128, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 150 * um, 100 * um, 0), complex_bits=64)
    G.propagate(1.0)
    assert O.rel_l2(H(G.field), golden["grid_in"]) < 1e-5
    G.expand(2 * mm)
    assert G.npoints == int(golden["grid_expand_n"]) and G.area_size == 2 * mm
    assert G.dL == pytest.approx(1 * mm / 128)
    assert O.rel_l2(H(G.field), golden["grid_expand_field"]) < 1e-5
    assert O.rel_l2(H(G.spectrum), golden["grid_expand_spectrum"]) < 1e-5
    G.coarse(2)
    assert G.npoints == int(golden["grid_coarse_n"])
    assert O.rel_l2(H(G.field), golden["grid_coarse_field"]) < 1e-5
    assert O.rel_l2(H(G.spectrum), golden["grid_coarse_spectrum"]) < 1e-5
    G.propagate(0.5)                       # the new grid propagates like any other
    g = O.grids(2 * mm, 128, 632 * nm)
    _, ref = O.propagate(np.fft.fft2(golden["grid_coarse_field"]), g["Kz"], 0.5)
    assert O.rel_l2(H(G.field), ref) < 1e-5


@pytest.mark.parametrize("n_in,n_out", [(1, 3), (100, 300), (2048, 4096), (64, 64)])
def test_expand_kernel_edge_padding(lp, n_in, n_out):
    """lp_expand is np.pad(mode="edge") exactly (beam2d.py:386-402), any size."""
    from lightprop2d_gb300 import backend as B
    rng = np.random.default_rng(n_in + n_out)
    x = (rng.normal(size=(n_in, n_in)) + 1j * rng.normal(size=(n_in, n_in))).astype(np.complex64)
    got = H(B.expand(torch.as_tensor(x, device="cuda"), n_out))
    d = (n_out - n_in) // 2
    assert np.array_equal(got, np.pad(x, d, mode="edge"))


@pytest.mark.parametrize("n,area_out,n_out", [(256, 0.5, 128), (256, 0.6, 0), (1024, 0.3, 512)])
def test_crop_vs_oracle(lp, n, area_out, n_out):
    area = 1.0 * mm
    x = (O.gaussian(n, area, 1.0, 0.2 * mm) * np.exp(1j * O.gaussian(n, area, 2.0, 0.3 * mm)))
    b = lp.Beam2D(area, n, 632 * nm, init_field=x)
    X = b.X.copy()
    xf = H(b.field).astype(np.complex128)
    b.crop(area_out * mm, n_out)
    m = n_out or n
    assert b.npoints == m and b.area_size == area_out * mm
    ref = O.crop(xf, X, area_out * mm, m, area_out * mm)
    assert O.rel_l2(H(b.field), ref) < 1e-6
    assert O.rel_l2(H(b.spectrum), np.fft.fft2(ref)) < 1e-5


@pytest.mark.parametrize("l1,l2", [(-2.0, 1.0), (3.0, 2.0), (5.0, 5.0)])
def test_lens_image_vs_oracle(lp, l1, l2):
    n, area, wl = 256, 1 * mm, 632 * nm
    x = O.gaussian(n, area, 1.0, 0.15 * mm) * np.exp(1j * O.gaussian(n, area, 1.5, 0.2 * mm))
    b = lp.Beam2D(area, n, wl, init_field=x)
    X = b.X.copy()
    xf = H(b.field).astype(np.complex128)
    b.lens_image(10.0, l1, l2)
    ref = O.lens_image(xf, X, 1 / wl, l1, l2)
    assert O.rel_l2(H(b.field), ref) < 1e-5
    s = -l1 / l2
    assert np.allclose(b.X, X * s)
    if s > 0:
        # a later lens follows the scaled grid, as in the reference
        b.lens(4.0)
        Xs = X * s
        fl, _ = O.lens(ref, Xs, Xs.reshape((-1, 1)), 1 / wl, 4.0)
        assert O.rel_l2(H(b.field), fl) < 1e-5


def test_grid_errors(lp):
    b = lp.Beam2D(1 * mm, 128, 632 * nm, init_field=np.ones((128, 128)))
    with pytest.raises(ValueError):
        b.expand(0.5 * mm)
    with pytest.raises(ValueError):
        b.expand(40 * mm)                  # 5120 points: not a supported size
    with pytest.raises(ValueError):
        b.coarse(3)
    with pytest.raises(ValueError):
        b.crop(1e-9)
