"""Workloads built on the differentiable kernels.

* ``spot_target`` / ``design_phase_mask``: phase-mask inverse design -- a
  learnable FP32 phase mask multiplies an input field, the result propagates
  a distance z, and Adam fits the output intensity to a target made of
  Gaussian spots.  Gradients come from the adjoint kernel.
* ``gaussian_screens``: seeded Gaussian random phase screens with a Gaussian
  spectrum (given correlation length and RMS phase) for split-step chains.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import autograd as A


def _grid(n, area, device):
    dL = area / n
    x = (torch.arange(-n // 2, n // 2, device=device, dtype=torch.float64) * dL)
    return x.reshape(1, -1), x.reshape(-1, 1)


def gaussian_field(n, area, waist, device="cuda"):
    """exp(-(x^2+y^2)/waist^2) on the Beam2D grid, complex64."""
    X, Y = _grid(n, area, device)
    return torch.exp(-(X ** 2 + Y ** 2) / waist ** 2).to(torch.complex64)


def spot_target(n, area, n_spots=16, waist=20e-4, seed=0, device="cuda", fill=0.6):
    """Sum of ``n_spots`` Gaussian intensity spots (1/e^2 waist ``waist``) at
    seeded random positions inside the central ``fill`` of the window."""
    rng = np.random.default_rng(seed)
    X, Y = _grid(n, area, device)
    pos = (rng.uniform(-0.5, 0.5, size=(n_spots, 2)) * fill * area)
    t = torch.zeros((n, n), dtype=torch.float64, device=device)
    for px, py in pos:
        t += torch.exp(-2 * ((X - px) ** 2 + (Y - py) ** 2) / waist ** 2)
    return t.to(torch.float32)


def design_phase_mask(n=1024, area=0.1, wl=1064e-7, waist=300e-4, z=10.0, steps=200,
                      lr=0.05, seed=0, n_spots=16, spot_waist=20e-4, device="cuda",
                      callback=None, graph: bool = False, timing: dict | None = None):
    """Fit a phase mask so that |P_z(E exp(i*phi))|^2 matches a spot target.

    Returns (phase, losses).  The loss is the mean squared difference between
    the output intensity and the target scaled to the same total power.

    ``graph=True`` captures one whole training step (forward kernels, loss,
    adjoint kernels, Adam) in a CUDA graph after three eager warm-up steps and
    replays it, so the host issues one launch per step.  ``timing`` (a dict)
    receives the device time per step of the loop, measured with CUDA events.
    """
    g = torch.Generator(device="cpu").manual_seed(seed)
    field = gaussian_field(n, area, waist, device)
    phase = (torch.rand((n, n), generator=g) * 2 * math.pi).to(device=device,
                                                                  dtype=torch.float32)
    phase.requires_grad_(True)
    target = spot_target(n, area, n_spots, spot_waist, seed, device)
    power = float((field.abs() ** 2).sum())
    target = target * (power / float(target.sum()))
    # Single-tensor Adam: its elementwise kernels spread the 1M-element mask
    # over the whole GPU, while the fused / foreach multi-tensor kernels give
    # one tensor 16 CTAs of 65536 elements (measured on GB300 at 1024^2:
    # 273 us of a 404 us graph-replayed step).
    kw = {"capturable": True} if graph else {}
    opt = torch.optim.Adam([phase], lr=lr, foreach=False, fused=False, **kw)
    losses = torch.empty(steps, dtype=torch.float32, device=device)

    def step():
        out = A.propagate(field, z, area, wl, phase=phase)
        loss = A.intensity_mse(out, target)    # mean((|out|^2 - target)^2)
        loss.backward()
        opt.step()
        return loss.detach()

    stream = torch.cuda.current_stream(device)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    if not graph:
        t0.record(stream)
        for it in range(steps):
            opt.zero_grad(set_to_none=True)
            losses[it] = step()                    # no host sync inside the loop
            if callback is not None:
                callback(it, float(losses[it]))
        t1.record(stream)
    else:
        side = torch.cuda.Stream(device=device)
        side.wait_stream(stream)
        warm = min(3, steps)
        with torch.cuda.stream(side):
            for it in range(warm):
                opt.zero_grad(set_to_none=False)
                losses[it] = step()
        stream.wait_stream(side)
        cg = torch.cuda.CUDAGraph()
        opt.zero_grad(set_to_none=False)
        with torch.cuda.graph(cg):
            opt.zero_grad(set_to_none=False)
            loss_static = step()
        t0.record(stream)
        for it in range(warm, steps):
            cg.replay()
            losses[it].copy_(loss_static)
            if callback is not None:
                callback(it, float(losses[it]))
        t1.record(stream)
    if timing is not None:
        torch.cuda.synchronize(device)
        done = steps if not graph else steps - min(3, steps)
        timing["ms_per_step"] = t0.elapsed_time(t1) / max(1, done)
    return phase.detach(), [float(v) for v in losses.cpu()]


def gaussian_screens(k, n, area, corr_len=200e-4, rms=1.0, seed=0, device="cuda"):
    """k seeded Gaussian random phase screens (float32, radians): white noise
    filtered by a Gaussian spectrum exp(-(2 pi f corr_len)^2 / 4) (a Gaussian
    autocorrelation of length ``corr_len``), scaled to RMS ``rms``."""
    from . import backend as B
    g = torch.Generator(device=device).manual_seed(seed)
    fx = np.fft.fftfreq(n, d=area / n)
    f2 = fx.reshape(1, -1) ** 2 + fx.reshape(-1, 1) ** 2
    filt = torch.as_tensor(np.exp(-(2 * math.pi) ** 2 * f2 * corr_len ** 2 / 4),
                           dtype=torch.float32, device=device)
    out = torch.empty((k, n, n), dtype=torch.float32, device=device)
    for i in range(k):
        w = torch.randn((n, n), generator=g, device=device).to(torch.complex64)
        spec = B.fft2(w)
        B.spectral_filter(spec, filt, field_out=w)
        s = w.real
        out[i] = s * (rms / s.std())
    return out
