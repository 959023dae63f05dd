"""GPU: 8192^2 grids (the reference's own performance script sweeps
npoints = 2048, 4096, 8192; tests/gaussbeam_performance.py:16).

At this size the numpy oracle would hold several GiB of complex128 and take
tens of seconds per transform, so the check restates the reference's
propagate (beam2d.py:485-490: fft2, H = exp(2*pi*i*(trunc(Kz z) - Kz z)) with
Kz in float64, ifft2) in torch complex128 on the device instead.  Bar: the
same relative-L2 1e-5 as every parity test."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
N, AREA, WL = 8192, 0.4, 632e-7
TOL = 1e-5


def _rel(a, b):
    return float(torch.linalg.vector_norm((a.to(torch.complex128) - b)) /
                 torch.linalg.vector_norm(b))


def _reference_propagate(x128, z):
    dL = AREA / N
    k = torch.fft.fftfreq(N, d=dL, dtype=torch.float64, device=x128.device)
    kz = torch.nan_to_num(torch.sqrt((1 / WL) ** 2 - k[None, :] ** 2 - k[:, None] ** 2))
    dk = kz * z
    H = torch.polar(torch.ones_like(dk), 2 * math.pi * (torch.trunc(dk) - dk))
    return torch.fft.ifft2(torch.fft.fft2(x128) * H)


def _gaussian(waist):
    x = (torch.arange(-N // 2, N // 2, dtype=torch.float64, device="cuda") * (AREA / N))
    return torch.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / waist ** 2).to(torch.complex128)


def test_fft2_8192_against_complex128():
    from lightprop2d_gb300 import backend as B
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.complex(torch.randn(N, N, device="cuda", generator=g),
                      torch.randn(N, N, device="cuda", generator=g))
    got = B.fft2(x)
    want = torch.fft.fft2(x.to(torch.complex128))
    assert _rel(got, want) < TOL
    del got, want


@pytest.mark.parametrize("z", [1.0, 20.0])
def test_propagate_field_8192_against_the_reference_sequence(z):
    from lightprop2d_gb300 import backend as B
    x = _gaussian(200e-4)
    got = B.propagate_field(x.to(torch.complex64), AREA, WL, z)
    want = _reference_propagate(x, z)
    assert _rel(got, want) < TOL
    e_in = float((x.abs() ** 2).sum())
    e_out = float((got.to(torch.complex128).abs() ** 2).sum())
    assert abs(e_out - e_in) < TOL * e_in


def test_beam2d_8192_lens_and_propagate():
    import lightprop2d_gb300 as lp
    x = _gaussian(300e-4)
    b = lp.Beam2D(AREA, N, WL, init_field=x.to(torch.complex64), complex_bits=64)
    b.lens(30.0)
    b.propagate(5.0)
    X = torch.arange(-N // 2, N // 2, dtype=torch.float64, device="cuda") * (AREA / N)
    lens = torch.polar(torch.ones(N, N, dtype=torch.float64, device="cuda"),
                       (X[None, :] ** 2 + X[:, None] ** 2) * (1 / WL) / (2 * 30.0))
    want = _reference_propagate(x * lens, 5.0)
    assert _rel(b.field, want) < TOL
