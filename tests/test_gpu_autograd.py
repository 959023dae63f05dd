"""GPU: gradients through the adjoint kernel vs torch.fft autograd (complex128)
and vs central finite differences of the kernel's own forward.

Bars: relative L2 <= 1e-4 against torch.fft autograd; <= 1e-3 against finite
differences (directional derivatives in float64 of the complex64 forward).
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def ref_propagate(u, z, area, wl, phase=None, after=False, kmask=None):
    """Reference forward in complex128 with torch.fft (differentiable)."""
    n = u.shape[0]
    dev = u.device
    dL = area / n
    f = torch.fft.fftfreq(n, d=dL, dtype=torch.float64, device=dev)
    kz2 = (1.0 / wl) ** 2 - f.reshape(1, -1) ** 2 - f.reshape(-1, 1) ** 2
    kz = torch.sqrt(torch.clamp(kz2, min=0.0))
    H = torch.exp(-2j * math.pi * kz * z)
    if kmask is not None:
        H = H * kmask.to(torch.complex128)
    x = u.to(torch.complex128)
    m = torch.exp(1j * phase.to(torch.float64)) if phase is not None else None
    if m is not None and not after:
        x = x * m
    y = torch.fft.ifft2(torch.fft.fft2(x) * H)
    if m is not None and after:
        y = y * m
    return y


def rel(a, b):
    a = a.detach().to(torch.complex128 if a.is_complex() else torch.float64)
    b = b.detach().to(torch.complex128 if b.is_complex() else torch.float64)
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def loss_fn(y, w, c):
    """A real loss touching |y|^2 and the complex value of y."""
    inten = y.real ** 2 + y.imag ** 2
    return (inten.double() * w).sum() + (y.to(torch.complex128) * c).real.sum()


def setup(n=256, seed=0):
    g = torch.Generator().manual_seed(seed)
    u = (torch.randn(n, n, generator=g) + 1j * torch.randn(n, n, generator=g)).to(torch.complex64)
    phase = torch.rand(n, n, generator=g) * 6.2831
    w = torch.rand(n, n, generator=g, dtype=torch.float64)
    c = torch.randn(n, n, generator=g, dtype=torch.complex128)
    return u.cuda(), phase.cuda().float(), w.cuda(), c.cuda()


@pytest.mark.parametrize("after", [False, True])
def test_grads_match_torch_fft_autograd(after):
    from lightprop2d_gb300 import autograd as A
    n, area, wl = 256, 0.05, 1064e-7
    u, phase, w, c = setup(n)
    z0 = 0.7
    # ours
    u1 = u.clone().requires_grad_(True)
    p1 = phase.clone().requires_grad_(True)
    z1 = torch.tensor(z0, dtype=torch.float64, device="cuda", requires_grad=True)
    y1 = A.propagate(u1, z1, area, wl, phase=p1, phase_after=after)
    loss_fn(y1, w, c).backward()
    # reference
    u2 = u.to(torch.complex128).clone().requires_grad_(True)
    p2 = phase.double().clone().requires_grad_(True)
    z2 = torch.tensor(z0, dtype=torch.float64, device="cuda", requires_grad=True)
    y2 = ref_propagate(u2, z2, area, wl, phase=p2, after=after)
    loss_fn(y2, w, c).backward()
    assert rel(y1, y2) < 1e-5
    assert rel(u1.grad, u2.grad) < 1e-4
    assert rel(p1.grad, p2.grad) < 1e-4
    assert abs(float(z1.grad) - float(z2.grad)) / abs(float(z2.grad)) < 1e-4


def test_grads_with_lens_and_kmask():
    from lightprop2d_gb300 import autograd as A
    n, area, wl, f = 128, 0.04, 632e-7, 2.0
    u, phase, w, c = setup(n, seed=3)
    km = torch.rand(n, n, device="cuda") * 0.5 + 0.5
    u1 = u.clone().requires_grad_(True)
    p1 = phase.clone().requires_grad_(True)
    y1 = A.propagate(u1, 0.4, area, wl, phase=p1, lens_f=f, kmask=km)
    loss_fn(y1, w, c).backward()
    # the lens is exp(i*(X^2+Y^2)*k0/(2f)): fold it into the reference phase
    dL = area / n
    x = torch.arange(-n // 2, n // 2, device="cuda", dtype=torch.float64) * dL
    lens_phase = (x.reshape(1, -1) ** 2 + x.reshape(-1, 1) ** 2) * (1 / wl) / (2 * f)
    p2 = phase.double().clone().requires_grad_(True)
    u2 = u.to(torch.complex128).clone().requires_grad_(True)
    y2 = ref_propagate(u2, 0.4, area, wl, phase=p2 + lens_phase, kmask=km)
    loss_fn(y2, w, c).backward()
    assert rel(y1, y2) < 1e-5
    assert rel(u1.grad, u2.grad) < 1e-4
    assert rel(p1.grad, p2.grad) < 1e-4


def test_phase_gradient_vs_finite_difference():
    from lightprop2d_gb300 import autograd as A
    n, area, wl, z = 256, 0.1, 1064e-7, 10.0
    u, phase, w, c = setup(n, seed=1)
    p = phase.clone().requires_grad_(True)
    loss_fn(A.propagate(u, z, area, wl, phase=p), w, c).backward()
    d = torch.randn(n, n, device="cuda", dtype=torch.float32,
                    generator=torch.Generator(device="cuda").manual_seed(7))
    # four-point central difference: truncation O(eps^4), and a step large
    # enough that the loss difference stands well above the complex64
    # forward's rounding (~1e-4 absolute on a loss of ~6e4)
    eps = 5e-2

    def f(t):
        with torch.no_grad():
            return loss_fn(A.propagate(u, z, area, wl, phase=phase + t * eps * d), w, c)
    fd = float((8 * (f(1) - f(-1)) - (f(2) - f(-2))) / (12 * eps))
    an = float((p.grad.double() * d.double()).sum())
    assert abs(fd - an) / abs(an) < 1e-3


def test_z_gradient_vs_finite_difference():
    from lightprop2d_gb300 import autograd as A
    n, area, wl = 256, 0.1, 632e-7
    u, phase, w, c = setup(n, seed=2)
    z = torch.tensor(3.0, dtype=torch.float64, device="cuda", requires_grad=True)
    loss_fn(A.propagate(u, z, area, wl, phase=phase), w, c).backward()
    h = 3e-7  # carrier phase step 2*pi*k0*h ~ 0.03 rad: truncation ~(k h)^2/6 ~ 1.5e-4
    with torch.no_grad():
        lp = loss_fn(A.propagate(u, 3.0 + h, area, wl, phase=phase), w, c)
        lm = loss_fn(A.propagate(u, 3.0 - h, area, wl, phase=phase), w, c)
    fd = float((lp - lm) / (2 * h))
    assert abs(fd - float(z.grad)) / abs(fd) < 1e-3


@pytest.mark.parametrize("every", [1, 4, 12])
def test_split_step_chain_gradients(every):
    from lightprop2d_gb300 import autograd as A
    from lightprop2d_gb300 import design as D
    n, area, wl, dz, K = 128, 0.05, 1550e-7, 0.5, 12
    u, _, w, c = setup(n, seed=4)
    screens = D.gaussian_screens(K, n, area, corr_len=20e-4, rms=1.0, seed=5)
    s1 = screens.clone().requires_grad_(True)
    u1 = u.clone().requires_grad_(True)
    y1 = A.split_step_chain(u1, s1, dz, area, wl, checkpoint_every=every)
    loss_fn(y1, w, c).backward()
    s2 = screens.double().clone().requires_grad_(True)
    u2 = u.to(torch.complex128).clone().requires_grad_(True)
    y2 = u2
    for k in range(K):
        y2 = ref_propagate(y2, dz, area, wl, phase=s2[k], after=True)
    loss_fn(y2, w, c).backward()
    assert rel(y1, y2) < 1e-5
    assert rel(u1.grad, u2.grad) < 1e-4
    assert rel(s1.grad, s2.grad) < 1e-4


def test_gaussian_screens_statistics():
    from lightprop2d_gb300 import design as D
    s = D.gaussian_screens(3, 256, 0.5, corr_len=200e-4, rms=1.0, seed=0)
    assert s.shape == (3, 256, 256) and s.dtype == torch.float32
    assert torch.allclose(s.std(dim=(1, 2)), torch.ones(3, device="cuda"), rtol=1e-3)
    # correlation length: neighbouring pixels (dL = 19.5 um << 200 um) are strongly correlated
    r = float((s[:, :, 1:] * s[:, :, :-1]).mean() / (s * s).mean())
    assert r > 0.95


def test_inverse_design_reduces_loss():
    from lightprop2d_gb300 import design as D
    phase, losses = D.design_phase_mask(n=256, area=0.1, wl=1064e-7, waist=300e-4, z=10.0,
                                        steps=40, lr=0.1, seed=0, spot_waist=40e-4)
    assert phase.shape == (256, 256)
    assert losses[-1] < 0.7 * losses[0]


def test_intensity_mse_matches_torch():
    """The fused loss kernel and its gradient against the same loss written
    in torch (float64 reference)."""
    from lightprop2d_gb300 import autograd as A
    rng = np.random.default_rng(7)
    for n in (64, 1024):
        y0 = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
        t = rng.uniform(0, 2, (n, n)).astype(np.float32)
        y = torch.as_tensor(y0, device="cuda").requires_grad_(True)
        tt = torch.as_tensor(t, device="cuda")
        loss = A.intensity_mse(y, tt)
        (3.0 * loss).backward()
        yr = torch.as_tensor(y0.astype(np.complex128)).requires_grad_(True)
        ref = ((yr.real ** 2 + yr.imag ** 2 - torch.as_tensor(t, dtype=torch.float64)) ** 2).mean()
        (3.0 * ref).backward()
        assert abs(float(loss.detach()) - float(ref.detach())) <= 1e-6 * abs(float(ref.detach()))
        g = y.grad.cpu().numpy()
        gr = yr.grad.numpy()
        assert np.linalg.norm(g - gr) <= 1e-5 * np.linalg.norm(gr)


def test_inverse_design_graph_matches_eager():
    """The CUDA-graph training step replays the same computation as eager."""
    from lightprop2d_gb300 import design as D
    kw = dict(n=256, area=0.1, wl=1064e-7, waist=300e-4, z=10.0, steps=12, lr=0.1, seed=1,
              spot_waist=40e-4)
    pe, le = D.design_phase_mask(**kw)
    pg, lg = D.design_phase_mask(**kw, graph=True)
    assert np.allclose(le, lg, rtol=1e-4), (le, lg)
    assert torch.allclose(pe, pg, rtol=1e-4, atol=1e-4)
