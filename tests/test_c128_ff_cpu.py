"""CPU: the complex128 family's float-float arithmetic (lp_c128_lines.cuh)
restated in numpy operation by operation -- the integer-bit conversions
between double and float-float (d2ff, f2d), the pair add and multiply, the
complex twiddle product, and zcis_2pi (cos and sin of 2 pi f by quarter-turn
reduction and Taylor series) -- against float64.

This pins the precision design without a GPU: a double survives the
conversion to 2^-47 relative over FP32's exponent range, the arithmetic
stays within ~4e-14 and the cos/sin within 1e-14 of float64 (the lens phase
too, whatever its size, through the double-double 1/(2 pi)), and values
outside the range flush or saturate as the header documents.  FMA is restated exactly: a
float32 product is exact in float64, so float32(a*b + c) computed in float64
is the fused result to within one float32 rounding of the low part.
"""
import numpy as np
import pytest

f32 = np.float32
u32, u64 = np.uint32, np.uint64


def fma(a, b, c):
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(f32)


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def ff_add2(ah, al, bh, bl):
    s, e = two_sum(ah, bh)
    return fast_two_sum(s, f32(e + f32(al + bl)))


def ff_mul2(ah, al, bh, bl):
    p = f32(ah * bh)
    return fast_two_sum(p, fma(ah, bl, fma(al, bh, fma(ah, bh, -p))))


def d2ff(d):
    """d2ff of the kernels: integer operations on the double's bits."""
    d = np.asarray(d, dtype=np.float64)
    b = d.view(u64)
    w1 = (b >> u64(32)).astype(u32)
    w0 = (b & u64(0xFFFFFFFF)).astype(u32)
    sgn = w1 & u32(0x80000000)
    e = ((w1 >> u32(20)) & u32(0x7FF)).astype(np.int64) - 1023
    lo = sgn.copy()
    hi = np.where(e < -126, sgn, u32(0))
    big = e > 127
    nan = big & (e == 1024) & (((w1 & u32(0xFFFFF)) | w0) != 0)
    hi = np.where(big, np.where(nan, u32(0x7FC00000), sgn | u32(0x7F800000)), hi)
    norm = (e >= -126) & (e <= 127)
    en = np.clip(e + 127, 0, 255).astype(u32)
    hi = np.where(norm, sgn | (en << u32(23)) | ((w1 & u32(0xFFFFF)) << u32(3)) | (w0 >> u32(29)),
                  hi)
    r = w0 & u32(0x1FFFFFFF)
    p = np.where(r > 0, np.floor(np.log2(np.maximum(r, 1))).astype(np.int64), 0)
    el = e - 52 + p
    sh_r = np.clip(p - 23, 0, 31).astype(u32)
    sh_l = np.clip(23 - p, 0, 31).astype(u32)
    mr = np.where(p >= 23, r >> sh_r, r << sh_l) & u32(0x7FFFFF)
    ok = norm & (r > 0) & (el >= -126)
    lo = np.where(ok, sgn | (np.clip(el + 127, 0, 255).astype(u32) << u32(23)) | mr, lo)
    return hi.view(f32), lo.view(f32)


def f2d(f):
    return np.asarray(f, dtype=f32).astype(np.float64)  # exact (normal floats)


def ff2d(h, l):
    return f2d(h) + f2d(l)


def inv_fact(n):
    v = 1.0 / float(np.prod(np.arange(1, n + 1, dtype=np.float64)))
    h = f32(v)
    return h, f32(v - np.float64(h))


HALF_PI = np.pi / 2


def zcis_2pi(f):
    """zcis_2pi of the kernels, on an array of doubles f."""
    f4 = 4.0 * np.asarray(f, dtype=np.float64)
    qd = np.rint(f4)
    rh, rl = d2ff(f4 - qd)                        # exact remainder, |rho| <= 1/2
    q = qd
    hp_h = f32(HALF_PI)
    hp_l = f32(HALF_PI - np.float64(hp_h))
    th, tl = ff_mul2(rh, rl, hp_h, hp_l)
    sh, sl = ff_mul2(th, tl, th, tl)
    i = lambda n: inv_fact(n)[0]
    ts = fma(fma(fma(i(17), sh, -i(15)), sh, i(13)), sh, -i(11))
    tc = fma(fma(fma(fma(-i(18), sh, i(16)), sh, -i(14)), sh, i(12)), sh, -i(10))

    def horner(acc, sign, n):
        ch, cl = (f32(1.0), f32(0.0)) if n == 0 else inv_fact(n)
        ph, pl = ff_mul2(sh, sl, acc[0], acc[1])
        return ff_add2(f32(sign * ch), f32(sign * cl), ph, pl)

    sa = (ts, np.zeros_like(ts))
    for sign, n in ((1, 9), (-1, 7), (1, 5), (-1, 3), (1, 0)):
        sa = horner(sa, sign, n)
    ca = (tc, np.zeros_like(tc))
    for sign, n in ((1, 8), (-1, 6), (1, 4), (-1, 2), (1, 0)):
        ca = horner(ca, sign, n)
    snh, snl = ff_mul2(th, tl, sa[0], sa[1])
    c, s = ff2d(*ca), ff2d(snh, snl)
    k = q.astype(np.int64) & 3
    cos = np.select([k == 0, k == 1, k == 2], [c, -s, -c], s)
    sin = np.select([k == 0, k == 1, k == 2], [s, c, -s], -c)
    return cos, sin


def test_d2ff_round_trip_over_fp32_range():
    rng = np.random.default_rng(0)
    d = rng.standard_normal(200000) * np.exp(rng.uniform(-60, 60, 200000))
    h, l = d2ff(d)
    back = ff2d(h, l)
    assert np.all(np.abs(back - d) <= 2.0 ** -47 * np.abs(d))
    assert np.all(np.abs(l) < np.abs(h) * 2.0 ** -23)          # non-overlapping pair
    assert np.array_equal(np.signbit(h), np.signbit(d))


def test_d2ff_edges():
    d = np.array([0.0, -0.0, 1e-40, -1e-40, 2.0 ** -110, 1e39, -np.inf, np.nan, 1.0,
                  np.nextafter(1.0, 2.0)])
    h, l = d2ff(d)
    assert h[0] == 0 and h[1] == 0 and np.signbit(h[1])          # signed zeros
    assert h[2] == 0 and h[3] == 0 and np.signbit(h[3])          # below 2^-126: flush
    assert h[4] == f32(2.0 ** -110) and l[4] == 0                  # low half underflows
    assert np.isposinf(h[5]) and np.isneginf(h[6]) and np.isnan(h[7])
    assert ff2d(h[8], l[8]) == 1.0
    assert ff2d(h[9], l[9]) - 1.0 == pytest.approx(2.0 ** -52, rel=1e-9)


def two_prod64(a, b):
    """Exact float64 product p + e (Dekker's splitting), the fma(a, b, -p) of
    the kernels' double-double step."""
    def split(x):
        c = 134217729.0 * x
        h = c - (c - x)
        return h, x - h
    p = a * b
    ah, al = split(a)
    bh, bl = split(b)
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def test_pair_arithmetic_and_twiddle_product():
    rng = np.random.default_rng(1)
    a, b, c, w = (rng.standard_normal(100000) for _ in range(4))
    ah, al = d2ff(a)
    bh, bl = d2ff(b)
    # each input converts within 2^-47, each operation adds ~2^-47
    assert np.max(np.abs(ff2d(*ff_add2(ah, al, bh, bl)) - (a + b)) /
                  (np.abs(a) + np.abs(b))) < 6e-14
    assert np.max(np.abs(ff2d(*ff_mul2(ah, al, bh, bl)) - a * b) / np.abs(a * b)) < 6e-14
    # complex twiddle product (zf_mul): re = a.re w.re - a.im w.im
    ch, cl = d2ff(c)
    wh, wl = d2ff(w)
    p1 = f32(ah * ch)
    p2 = f32(bh * wh)
    e1 = fma(ah, cl, fma(al, ch, fma(ah, ch, -p1)))
    e2 = fma(bh, wl, fma(bl, wh, fma(bh, wh, -p2)))
    s, t = two_sum(p1, -p2)
    rh, rl = fast_two_sum(s, f32(t + f32(e1 - e2)))
    want = a * c - b * w
    assert np.max(np.abs(ff2d(rh, rl) - want) / (np.abs(a * c) + np.abs(b * w))) < 6e-14


def test_zcis_2pi_against_float64():
    rng = np.random.default_rng(2)
    f = np.concatenate([-rng.uniform(0.0, 1.0, 200000),
                        np.array([0.0, -0.125, -0.25, -0.375, -0.5, -0.75, -1 + 1e-16]),
                        rng.uniform(-3.0, 3.0, 20000)])
    c, s = zcis_2pi(f)
    ang = 2 * np.pi * f
    assert np.max(np.abs(c - np.cos(ang))) < 1e-14
    assert np.max(np.abs(s - np.sin(ang))) < 1e-14


def test_lens_phase_turns_double_double():
    """zxmul_ff: the reference's float64 phase turned into turns by the
    double-double 1/(2 pi); cos/sin then agree with float64 cos/sin of the
    phase to the phase's own rounding."""
    inv_h, inv_l = 0.15915494309189535, -9.839338337591243e-18
    ph = np.random.default_rng(3).uniform(0, 2e3, 50000)
    p, e = two_prod64(ph, np.full_like(ph, inv_h))
    e = e + ph * inv_l
    c, s = zcis_2pi((p - np.rint(p)) + e)
    assert np.max(np.abs(c - np.cos(ph))) < 2e-14
    assert np.max(np.abs(s - np.sin(ph))) < 2e-14
