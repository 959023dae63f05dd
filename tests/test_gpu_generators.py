"""GPU: profile generators evaluated inside the first FFT pass (compact
2N tables, no N x N mask) match the reference's host-mask semantics."""
import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm = O.um, O.nm, O.mm
TOL = 1e-5


@pytest.fixture(scope="module")
def lp():
    import lightprop2d_gb300 as lp
    return lp


def H(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def cases(lp, A):
    return [(lp.round_hole, (0.21 * A, 0.05 * A, -0.03 * A)),
            (lp.round_hole, (0.25 * A,)),
            (lp.rectangle_hole, (0.3 * A, 0.2 * A, 0.02 * A, 0.01 * A)),
            (lp.square_hole, (0.33 * A,)),
            (lp.square_slits, (0.1 * A, 0.4 * A)),
            (lp.gaussian_beam, (1.3, 0.2 * A, 0.03 * A, -0.05 * A)),
            (lp.plane_wave, ())]


@pytest.mark.parametrize("n", [256, 2048])
def test_coordinate_filter_generators_fused(lp, n):
    from lightprop2d_gb300 import generators as G
    A, wl, z = 1 * mm, 632 * nm, 0.7
    x = O.random_phase_hole(n, A, 0.45 * A, seed=n)
    g = O.grids(A, n, wl)
    for f, args in cases(lp, A):
        b = lp.Beam2D(A, n, wl, init_field=x, complex_bits=64)
        Xr = b.X.copy()
        Yr = Xr.reshape((-1, 1))          # aliases Xr, as Beam2D's Y aliases X
        mask = np.broadcast_to(f(Xr, Yr, *args), (n, n))
        b.coordinate_filter(f_gen=f, fargs=args)
        assert isinstance(b._pend_xmask, G.GenMask), f.__name__
        assert np.array_equal(b.X, Xr)    # gaussian_beam's in-place grid shift
        b.propagate(z)
        fl = x.astype(np.complex64).astype(np.complex128) * mask
        _, ref = O.propagate(np.fft.fft2(fl), g["Kz"], z)
        assert O.rel_l2(H(b.field), ref) < TOL, f.__name__
        # and without a propagate: the field itself
        c = lp.Beam2D(A, n, wl, init_field=x, complex_bits=64)
        c.coordinate_filter(f_gen=f, fargs=args)
        assert O.rel_l2(H(c.field), fl) < 1e-6, f.__name__


def test_spectral_filter_generators_fused(lp):
    from lightprop2d_gb300 import generators as G
    n, A, wl = 512, 1 * mm, 632 * nm
    x = O.random_phase_hole(n, A, 0.3 * A, seed=3)
    g = O.grids(A, n, wl)
    for f, args in [(lp.rectangle_hole, (900.0, 600.0)), (lp.gaussian_beam, (1.0, 800.0)),
                    (lp.square_slits, (150.0, 700.0))]:
        b = lp.Beam2D(A, n, wl, init_field=x, complex_bits=64)
        Kx = b.Kx.copy()
        m = np.broadcast_to(f(Kx, Kx.reshape((-1, 1)), *args), (n, n))
        b.spectral_filter(f_gen=f, fargs=args)
        ref = np.fft.ifft2(np.fft.fft2(x.astype(np.complex64)) * m)
        assert O.rel_l2(H(b.field), ref) < TOL, f.__name__
    # round_hole on the K grid is not row-interval shaped: host mask path
    b = lp.Beam2D(A, n, wl, init_field=x, complex_bits=64)
    b.spectral_filter(f_gen=lp.round_hole, fargs=(700.0,))
    m = lp.round_hole(b.Kx.copy(), b.Kx.copy().reshape((-1, 1)), 700.0)
    assert O.rel_l2(H(b.field), np.fft.ifft2(np.fft.fft2(x.astype(np.complex64)) * m)) < TOL


def test_generator_mask_through_abi(lp):
    """Compact tables through the C ABI directly (lp_coordinate_filter)."""
    from lightprop2d_gb300 import backend as B, generators as G
    n, dL = 128, 1e-4
    X = np.arange(-n // 2, n // 2) * dL
    Y = X.reshape((-1, 1))
    gm = G.compact(lp.round_hole, (30 * dL, 3 * dL, -2 * dL), X, Y, "cuda")
    f = torch.ones((n, n), dtype=torch.complex64, device="cuda")
    B.coordinate_filter(f, gm)
    ref = lp.round_hole(X.copy(), X.copy().reshape((-1, 1)), 30 * dL, 3 * dL, -2 * dL)
    assert np.array_equal(H(f).real, ref.astype(np.float32))
    assert np.array_equal(H(G.dense(gm, n)), ref.astype(np.float32))
    with pytest.raises(ValueError):      # span tables are x-domain only
        B.propagate(torch.ones((n, n), dtype=torch.complex64, device="cuda"), n * dL, 632e-7,
                    1.0, kmask=gm)
