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


# ---------------------------------------------------------------------------
# Compact (2N-table) forms of the deterministic generators, which the first
# FFT pass evaluates on the device (lightprop2d_gb300.generators).
# ---------------------------------------------------------------------------
def _dense(f_gen, fargs, x, y):
    from lightprop2d_gb300 import generators as G
    gm = G.compact(f_gen, fargs, x, y, "cpu")
    assert gm is not None
    return G.dense(gm, x.size).numpy()


def _grid(n, dL):
    x = np.arange(-n // 2, n // 2, 1) * dL
    return x, x.reshape((-1, 1))


def test_compact_generators_match_reference_golden(golden):
    n, dL = 32, 1e-4
    cases = [(P.plane_wave, (), "prof_plane"),
             (P.round_hole, (8 * dL, 2 * dL, 0), "prof_round"),
             (P.rectangle_hole, (10 * dL, 6 * dL, dL, 0), "prof_rect"),
             (P.square_hole, (8 * dL,), "prof_square"),
             (P.square_slits, (4 * dL, 10 * dL), "prof_slits")]
    for f, args, key in cases:
        x, y = _grid(n, dL)
        assert np.array_equal(_dense(f, args, x, y), golden[key].astype(np.float32)), key
    x, y = _grid(n, dL)
    g = _dense(P.gaussian_beam, (1.5, 8 * dL, dL, -2 * dL), x.copy(), y.copy())  # as generated
    assert np.allclose(g, golden["prof_gauss"], rtol=2e-7, atol=1e-12)


@pytest.mark.parametrize("seed", range(6))
def test_compact_generators_match_dense_random(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.choice([64, 256, 1024]))
    dL = float(rng.uniform(0.5, 3)) * 1e-4
    A = n * dL
    R = float(rng.uniform(0.02, 0.4)) * A
    x0, y0 = (float(v) for v in rng.uniform(-0.2, 0.2, 2) * A)
    if seed % 2:  # grid-aligned parameters put points exactly on edges
        R, x0, y0 = 12 * dL, 3 * dL, -5 * dL
    for f, args in [(P.round_hole, (R, x0, y0)), (P.rectangle_hole, (R, 0.7 * R, x0, y0)),
                    (P.square_hole, (R, x0, y0)), (P.square_slits, (0.3 * R, R, x0, y0)),
                    (P.plane_wave, ())]:
        x, y = _grid(n, dL)
        ref = f(x.copy(), y.copy().reshape((-1, 1)), *args)
        ref = np.broadcast_to(ref, (n, n)).astype(np.float32)
        assert np.array_equal(_dense(f, args, x, y), ref), (f.__name__, n)
    # gaussian_beam: values to FP32 rounding, and the in-place grid shift
    x, y = _grid(n, dL)
    xr = x.copy()
    yr = xr.reshape((-1, 1))
    ref = P.gaussian_beam(xr, yr, 2.0, R, x0, y0)
    g = _dense(P.gaussian_beam, (2.0, R, x0, y0), x, y)
    assert np.allclose(g, ref, rtol=3e-7, atol=1e-30)
    assert np.array_equal(x, xr)


def test_compact_generators_on_fftfreq_grid():
    """Spectral masks: separable generators on the unshifted K grid."""
    n, dL = 128, 1e-4
    kx = np.fft.fftfreq(n, d=dL)
    ky = kx.reshape((-1, 1))
    for f, args in [(P.rectangle_hole, (800.0, 500.0)), (P.square_slits, (200.0, 900.0)),
                    (P.gaussian_beam, (1.0, 700.0))]:
        ref = f(kx.copy(), kx.copy().reshape((-1, 1)), *args)
        ref = np.broadcast_to(ref, (n, n)).astype(np.float32)
        got = _dense(f, args, kx.copy(), kx.copy().reshape((-1, 1)))
        assert np.allclose(got, ref, rtol=3e-7, atol=1e-30), f.__name__
    from lightprop2d_gb300 import generators as G
    assert G.compact(P.round_hole, (500.0,), kx, ky, "cpu", allow_span=False) is None
    assert G.compact(P.random_round_hole, (500.0,), kx, ky, "cpu") is None
