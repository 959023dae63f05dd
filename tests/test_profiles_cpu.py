"""CPU: profile generators vs the reference's outputs (golden vectors) and the
exact asserts of tests/test_profiles.py:31-38."""
import numpy as np
import pytest

from lightprop2d_gb300 import profiles as P


def grid(n=32, dL=1e-4):
    x = np.arange(-n // 2, n // 2, 1) * dL
    return x, x.reshape((-1, 1))


def test_against_reference(golden):
    dL = 1e-4
    x, y = grid()
    assert np.array_equal(P.plane_wave(x.copy(), y.copy()), golden["prof_plane"])
    assert np.array_equal(P.gaussian_beam(x.copy(), y.copy(), 1.5, 8 * dL, dL, -2 * dL),
                          golden["prof_gauss"])
    assert np.array_equal(P.round_hole(x.copy(), y.copy(), 8 * dL, 2 * dL, 0), golden["prof_round"])
    assert np.array_equal(P.rectangle_hole(x.copy(), y.copy(), 10 * dL, 6 * dL, dL, 0),
                          golden["prof_rect"])
    assert np.array_equal(P.square_hole(x.copy(), y.copy(), 8 * dL), golden["prof_square"])
    assert np.array_equal(P.square_slits(x.copy(), y.copy(), 4 * dL, 10 * dL), golden["prof_slits"])
    np.random.seed(5)
    assert np.array_equal(P.random_round_hole(x.copy(), y.copy(), 8 * dL), golden["prof_rand_round"])
    np.random.seed(5)
    assert np.array_equal(P.random_round_hole_bin(x.copy(), y.copy(), 8 * dL, 0, 0, 2),
                          golden["prof_rand_round_bin"])
    np.random.seed(5)
    assert np.allclose(P.random_round_hole_phase(x.copy(), y.copy(), 8 * dL),
                       golden["prof_rand_round_phase"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("npoints", [64, 256])
def test_reference_profile_asserts(npoints):
    dL = 1e-4
    x, y = grid(npoints, dL)
    R = d = rho0 = dL * npoints / 4
    A0 = 1.
    dx = dy = dL * npoints / 4
    assert P.gaussian_beam(x, y, A0, rho0)[npoints // 2, npoints // 2] == A0
    assert np.sum(P.plane_wave(x, y)) == npoints ** 2
    P.random_wave(x, y)
    P.round_hole(x, y, R)
    P.random_round_hole(x, y, R)
    assert np.allclose(P.square_hole(x, y, d), P.rectangle_hole(x, y, dx, dy))
    assert np.allclose(P.square_slits(x, y, d, d),
                       P.square_hole(x, y, d, x0=-d / 2) + P.square_hole(x, y, d, x0=d / 2))


def test_round_hole_radius_is_R_over_sqrt2():
    x, y = grid(256, 1e-4)
    R = 40e-4
    h = P.round_hole(x, y, R)
    r = np.sqrt(x ** 2 + y ** 2)
    assert r[h].max() <= R / np.sqrt(2) + 1e-12
    assert r[~h].min() > R / np.sqrt(2) - 1.5e-4


def test_gaussian_beam_shifts_args_in_place():
    x, y = grid(16, 1e-4)
    x0 = x.copy()
    P.gaussian_beam(x, y, 1.0, 1e-3, x0=2e-4)
    assert np.allclose(x, x0 - 2e-4)


def test_torch_inputs():
    torch = pytest.importorskip("torch")
    x, y = grid(32)
    xt, yt = torch.as_tensor(x), torch.as_tensor(y)
    assert np.allclose(P.gaussian_beam(xt.clone(), yt.clone(), 1, 5e-4).numpy(),
                       P.gaussian_beam(x.copy(), y.copy(), 1, 5e-4))
    assert np.array_equal(P.round_hole(xt, yt, 8e-4).numpy(), P.round_hole(x, y, 8e-4))
    assert np.array_equal(P.square_slits(xt, yt, 4e-4, 1e-3).numpy(),
                          P.square_slits(x, y, 4e-4, 1e-3))
