"""CPU: the kernels' phase arithmetic restated in numpy float32 operation by
operation -- the transfer-function phase of the column pass (column_constant
+ kz_phase_ff in lp_device.cuh, parameters as make_kparams in lp_capi.cu)
against the float64 phase Kz*z of the reference (beam2d.py:485-489), the
lens phase (lens_cycles, beam2d.py:508-511) and the reduction of FP32 phase
masks (cis_radians).

This pins the precision design without a GPU: the float-float phase stays
within 6e-8 cycles of float64 out to z = 50 cm (the float32 rounding of the
reduced phase, |f| <= 0.5, is itself up to 3e-8), near the evanescent
cut-off only with the renormalisation step, while plain FP32 loses the
phase.
FMA is restated exactly: a float32 product is exact in float64, so
float32(a*b + c) computed in float64 is the rounded fused result.
"""
import numpy as np
import pytest

f32 = np.float32


def fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def two_prod(a, b):
    p = (a * b).astype(f32)
    return p, fma(a, b, -p)


def two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    return s, ((a - (s - bb)) + (b - bb)).astype(f32)


def ff(d):
    hi = f32(d)
    return hi, f32(d - np.float64(hi))


def grid_terms(n, area, wl, z):
    """Per point (qx, qy) = (sx^2, sy^2) and the float-float beta and R."""
    dl = area / n
    val = 1.0 / (n * dl)
    s = np.fft.fftfreq(n, 1.0 / n).astype(np.int64)
    qx = np.broadcast_to((s[None, :] ** 2).astype(f32), (n, n))
    qy = np.broadcast_to((s[:, None] ** 2).astype(f32), (n, n))
    return qx, qy, ff((val * wl) ** 2), ff(z / wl)


def phase_ff(n, area, wl, z, renormalise=True):
    """Fractional phase (cycles) and evanescent mask as the kernel computes
    them (the rsqrt seed is exact here; the Newton step makes the result
    insensitive to the seed's few-ulp error on the device)."""
    qx, qy, (bh, bl), (rh, rl) = grid_terms(n, area, wl, z)
    bh, bl, rh, rl = (np.full((n, n), v, f32) for v in (bh, bl, rh, rl))
    th, tl = two_prod(bh, qx)                      # column_constant
    tl = fma(bl, qx, tl)
    ah, e = two_sum(np.ones_like(th), -th)
    al = (e - tl).astype(f32)
    uh, ul = two_prod(bh, qy)                      # kz_phase_ff
    ul = fma(bl, qy, ul)
    v0, e = two_sum(ah, -uh)
    if renormalise:
        vh, vl = two_sum(v0, (e + (al - ul)).astype(f32))
    else:
        vh, vl = v0, (e + (al - ul)).astype(f32)
    evan = ~(vh > 0)
    vv = np.where(evan, f32(1), vh).astype(f32)
    y = (1.0 / np.sqrt(vv.astype(np.float64))).astype(f32)
    s0 = (vv * y).astype(f32)
    r = (fma(-s0, s0, vv) + np.where(evan, f32(0), vl)).astype(f32)
    c = (r * (f32(0.5) * y)).astype(f32)
    ph, pe = two_prod(rh, s0)
    pl = (pe + fma(rh, c, (rl * s0).astype(f32))).astype(f32)
    return ((ph - np.rint(ph)).astype(f32) + pl).astype(f32), evan


def phase_fp32(n, area, wl, z):
    """The plain-FP32 comparison variant (kz_phase_f32)."""
    qx, qy, (bh, _), (rh, rl) = grid_terms(n, area, wl, z)
    v = (f32(1) - bh * (qx + qy).astype(f32)).astype(f32)
    evan = ~(v > 0)
    p = ((rh + rl) * np.sqrt(np.where(evan, f32(0), v))).astype(f32)
    return (p - np.rint(p)).astype(f32), evan


def phase_ref(n, area, wl, z):
    """Kz*z in float64 (beam2d.py:189-205, :485-489): Kz = sqrt(k0^2 - Kx^2 - Ky^2)."""
    kx = np.fft.fftfreq(n, area / n)
    k2 = (1.0 / wl) ** 2 - kx[None, :] ** 2 - kx[:, None] ** 2
    return np.sqrt(np.maximum(k2, 0.0)) * z, k2 <= 0


def max_err(f, evan, n, area, wl, z):
    ref, evan_ref = phase_ref(n, area, wl, z)
    ok = ~evan & ~evan_ref
    d = f.astype(np.float64) - ref
    d -= np.rint(d)
    return float(np.abs(d[ok]).max())


@pytest.mark.parametrize("z", [0.1, 1.0, 5.0, 10.0, 50.0])
def test_float_float_phase_config2(z):
    """2048^2, 2 mm, 632 nm: float-float within 6e-8 cycles at every z of
    the workload (measured 2.8e-8 at 0.1 cm to 4.2e-8 at 50 cm); plain FP32
    off by 1.7e-4 cycles at 0.1 cm and 7.7e-2 at 50 cm."""
    n, area, wl = 2048, 0.2, 632e-7
    f, evan = phase_ff(n, area, wl, z)
    assert max_err(f, evan, n, area, wl, z) < 6e-8
    g, evan32 = phase_fp32(n, area, wl, z)
    assert max_err(g, evan32, n, area, wl, z) > 1e-4


@pytest.mark.parametrize("n,area,wl,z", [
    (2048, 0.10409037570395337, 1064e-7, 1.7394964232143395),
    (2048, 0.04663, 632e-7, 1.87),
    (1024, 0.025, 532e-7, 12.0)])
def test_float_float_phase_near_cutoff(n, area, wl, z):
    """Grids whose spectrum reaches the evanescent cut-off: with the
    renormalisation of (v_hi, v_lo) the phase stays within 1e-7 cycles
    everywhere (measured 3e-8 to 5e-8); without it the one-step Newton square
    root loses 1e-3 to 2e-2 cycles next to the cut-off (the failure the
    renormalisation fixed)."""
    f, evan = phase_ff(n, area, wl, z)
    assert max_err(f, evan, n, area, wl, z) < 1e-7
    g, evan0 = phase_ff(n, area, wl, z, renormalise=False)
    assert max_err(g, evan0, n, area, wl, z) > 10 * max_err(f, evan, n, area, wl, z)


def test_lens_phase_float_float():
    """Lens phase kappa*(jx^2+jy^2) cycles (lens_cycles, set_lens): exact
    integer jx^2+jy^2, float-float kappa, against float64, at 2048^2, 2 mm,
    632 nm and f = 1 cm (about 13 cycles at the corner: 79 rad at r = 1 mm)."""
    n, area, wl, f = 2048, 0.2, 632e-7, 1.0
    dl = area / n
    kh, kl = ff(dl * dl * (1.0 / wl) / (4.0 * np.pi * f))
    j = np.arange(n, dtype=np.int64) - n // 2
    m64 = j[None, :] ** 2 + j[:, None] ** 2
    m = m64.astype(f32)
    assert np.array_equal(m.astype(np.int64), m64)                # exact integers
    khf, klf = np.full(m.shape, kh, f32), np.full(m.shape, kl, f32)
    c_hi, c_e = two_prod(khf, m)
    c_lo = fma(klf, m, c_e)
    got = ((c_hi - np.rint(c_hi)).astype(f32) + c_lo).astype(f32).astype(np.float64)
    ref = m64 * (dl * dl * (1.0 / wl) / (4.0 * np.pi * f))
    d = got - ref
    d -= np.rint(d)
    assert np.abs(d).max() < 6e-8


def test_cody_waite_phase_reduction():
    """cis_radians' reduction of an FP32 phase mask value to [-pi, pi]:
    r = fma(-k, lo, fma(-k, hi, phi)), k = rint(phi / 2pi), 2pi = hi + lo,
    stays within 2.5e-7 rad (about one ulp of pi) of the exact reduction for
    |phi| up to 1e4 rad."""
    rng = np.random.default_rng(3)
    phi = rng.uniform(-1e4, 1e4, 200000).astype(f32)
    hi, lo = ff(2 * np.pi)
    inv = f32(1 / (2 * np.pi))
    k = np.rint((phi * inv).astype(f32)).astype(f32)
    r = fma(-k, np.full_like(k, lo), fma(-k, np.full_like(k, hi), phi))
    exact = phi.astype(np.float64) - k.astype(np.float64) * 2 * np.pi
    assert np.abs(r.astype(np.float64) - exact).max() < 2.5e-7
    assert np.abs(r).max() <= np.pi + 1e-3
