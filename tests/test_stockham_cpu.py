"""CPU: the mixed-radix Stockham schedule of the 1-D transform
(lp_fft_core.cuh: Plan<N>, fft_first / fft_stage) restated in numpy and
checked against numpy.fft (the reference's _fft2 convention, beam2d.py:207-229).

Stage s with radix R and Ns = product of the earlier radices computes, for
each butterfly b < N/R,
    a[r] = x[b + r*N/R] * W_(Ns*R)^(r*(b mod Ns))           (r < R)
    y[(b/Ns)*Ns*R + (b mod Ns) + r*Ns] = DFT_R(a)[r]
with W_M = exp(-2*pi*i/M) forward.  In float64 the schedule reproduces the
DFT to round-off; with complex64 data and twiddles rounded to float32 from
double (fill_twiddles) it stays at the FP32 level.
"""
import numpy as np
import pytest

PLAN = {16: (16,), 32: (16, 2), 64: (16, 4), 128: (16, 8), 256: (16, 16), 512: (16, 16, 2),
        1024: (16, 16, 4), 2048: (16, 16, 8), 4096: (16, 16, 16), 8192: (16, 16, 16, 2)}


def stockham(x, sign=-1, dtype=np.complex128):
    """Forward (sign -1) or unscaled inverse (+1) transform of the last axis."""
    x = np.asarray(x, dtype=dtype)
    n = x.shape[-1]
    ns = 1
    for R in PLAN[n]:
        nb = n // R
        b = np.arange(nb)
        k = b % ns
        r = np.arange(R)
        a = x[..., b[None, :] + r[:, None] * nb]                       # (..., R, nb)
        if ns > 1:                                                     # stage twiddles
            w = np.exp(sign * 2j * np.pi * (r[:, None] * k[None, :]) / (ns * R))
            a = a * w.astype(dtype)
        dft = np.exp(sign * 2j * np.pi * np.outer(r, r) / R).astype(dtype)
        yr = np.einsum("rq,...qb->...rb", dft, a)                      # DFT_R per butterfly
        out = np.empty_like(x)
        idx = (b // ns)[None, :] * ns * R + k[None, :] + r[:, None] * ns
        out[..., idx] = yr
        x = out
        ns *= R
    return x


@pytest.mark.parametrize("n", sorted(PLAN))
def test_schedule_is_the_dft(n):
    rng = np.random.default_rng(n)
    x = rng.normal(size=(3, n)) + 1j * rng.normal(size=(3, n))
    ref = np.fft.fft(x)
    assert np.abs(stockham(x) - ref).max() <= 1e-12 * np.abs(ref).max()
    inv = stockham(ref, sign=+1) / n
    assert np.abs(inv - x).max() <= 1e-12 * np.abs(x).max()


@pytest.mark.parametrize("n", [256, 2048, 4096])
def test_schedule_complex64_accuracy(n):
    """complex64 data and float32 twiddles: rel-L2 at the FP32 level."""
    rng = np.random.default_rng(n + 1)
    x = (rng.normal(size=(4, n)) + 1j * rng.normal(size=(4, n))).astype(np.complex64)
    got = stockham(x, dtype=np.complex64)
    ref = np.fft.fft(x.astype(np.complex128))
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6
