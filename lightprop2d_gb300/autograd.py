"""Differentiable propagation on the GB300 kernels.

``propagate`` is a ``torch.autograd.Function`` around the fused field -> field
kernel sequence:

    y = P_z(u * m)        (mask before propagation, the default), or
    y = m * P_z(u)        (``phase_after=True``: propagate, then screen)

with ``P_z = F^-1 diag(kmask * H(z)) F`` and ``m = exp(i*phase) * lens``.  Its
backward is the hand-written adjoint kernel (``LP_FLAG_ADJOINT``):

    grad_u     = conj(m) * P_z^H(grad_y)          (pre-multiply case)
    grad_phase = Im(conj(x) * grad_x)             x = the multiplied field
    grad_z     = Re <grad_y, dy/dz>,  dy/dz from the LP_FLAG_DZ kernel

(PyTorch's complex convention: a linear map's backward is its adjoint.)

``split_step_chain`` runs K alternating propagate / phase-screen steps and
backpropagates through them without storing every field: it keeps one field
per ``checkpoint_every`` steps and recomputes each segment during backward.
"""
from __future__ import annotations

import torch

from . import _lib as L
from . import backend as B


def _z_value(z) -> float:
    return float(z.detach()) if isinstance(z, torch.Tensor) else float(z)


class _Propagate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, field, phase, z, area_size, wl, lens_f, kmask, after):
        zv = _z_value(z)
        flags = L.LP_FLAG_XMASK_AFTER if after else 0
        out = B.propagate_field(field.contiguous(), area_size, wl, zv, lens_f=lens_f,
                                xmask=phase, xmask_phase=phase is not None, kmask=kmask,
                                flags=flags)
        ctx.geom = (area_size, wl, zv, lens_f, after, phase is not None)
        ctx.z_dtype = z.dtype if isinstance(z, torch.Tensor) else torch.float64
        ctx.kmask = kmask
        ctx.save_for_backward(field, phase if phase is not None else field.new_empty(0), out)
        return out

    @staticmethod
    def backward(ctx, gy):
        field, phase, out = ctx.saved_tensors
        area, wl, zv, lens_f, after, has_phase = ctx.geom
        phase = phase if has_phase else None
        kmask = ctx.kmask
        gy = gy.contiguous()
        if gy.dtype != torch.complex64:
            gy = gy.to(torch.complex64)
        need_u, need_phi, need_z = ctx.needs_input_grad[:3]
        after_flag = L.LP_FLAG_XMASK_AFTER if after else 0
        grad_u = grad_phi = grad_z = None
        if need_u or (need_phi and not after):
            grad_u = B.propagate_field(gy, area, wl, zv, lens_f=lens_f, xmask=phase,
                                       xmask_phase=has_phase, kmask=kmask,
                                       flags=L.LP_FLAG_ADJOINT | after_flag)
        if need_phi:
            # Im(conj(x) * grad_x) at the multiplied field x:
            #   before propagation x = u*m, grad_x = conj(m)... -> Im(conj(u) grad_u)
            #   after propagation  x = y,   grad_x = grad_y
            grad_phi = (B.phase_grad(field.contiguous(), grad_u) if not after
                        else B.phase_grad(out, gy))
        if need_z:
            dydz = B.propagate_field(field.contiguous(), area, wl, zv, lens_f=lens_f,
                                     xmask=phase, xmask_phase=has_phase, kmask=kmask,
                                     flags=L.LP_FLAG_DZ | after_flag)
            g = torch.vdot(gy.reshape(-1), dydz.reshape(-1)).real
            grad_z = g.to(ctx.z_dtype)
        return (grad_u if need_u else None), grad_phi, grad_z, None, None, None, None, None


class _IntensityMSE(torch.autograd.Function):
    """mean((|y|^2 - target)^2) in one reduction kernel; its gradient
    4/count * (|y|^2 - target) * y in one elementwise kernel (the upstream
    gradient is read on the device, so the step stays graph-capturable)."""

    @staticmethod
    def forward(ctx, y, target):
        ctx.save_for_backward(y, target)
        s = B.intensity_mse_sum(y, target)
        return (s / y.numel()).to(torch.float32).reshape(())

    @staticmethod
    def backward(ctx, g):
        y, target = ctx.saved_tensors
        up = g.reshape(1).to(torch.float32).contiguous()
        return B.intensity_mse_grad(y, target, up, 4.0 / y.numel()), None


def intensity_mse(y: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """Differentiable mean((|y|^2 - target)^2) for complex64 y and float32
    target of the same shape (library kernels for the value and gradient)."""
    if y.dtype != torch.complex64:
        raise ValueError("y must be complex64")
    return _IntensityMSE.apply(y.contiguous(), target.to(torch.float32).contiguous())


def propagate(field: torch.Tensor, z, area_size: float, wl: float, phase=None,
              lens_f: float = 0.0, kmask=None, phase_after: bool = False) -> torch.Tensor:
    """Differentiable fused propagate (field, phase mask and z gradients).

    field: complex64 CUDA (N, N).  phase: float32 (N, N) radians or None.
    z: float, or a 0-d tensor when its gradient is wanted.  kmask: optional
    constant spectral multiplier.  phase_after: apply exp(i*phase) after the
    propagation instead of before.
    """
    if field.dtype != torch.complex64:
        field = field.to(torch.complex64)
    if phase is not None and phase.dtype != torch.float32:
        raise ValueError("phase must be float32")
    return _Propagate.apply(field, phase, z, float(area_size), float(wl), float(lens_f), kmask,
                            bool(phase_after))


class _Chain(torch.autograd.Function):
    """u_{k+1} = exp(i*screens[k]) * P_dz(u_k), k = 0..K-1."""

    @staticmethod
    def forward(ctx, field, screens, dz, area_size, wl, every):
        K = screens.shape[0]
        u = field.contiguous()
        ckpts = []
        for k in range(K):
            if k % every == 0:
                ckpts.append(u)
            u = B.propagate_field(u, area_size, wl, dz, xmask=screens[k], xmask_phase=True,
                                  flags=L.LP_FLAG_XMASK_AFTER)
        ctx.geom = (dz, area_size, wl, every, K)
        ctx.save_for_backward(screens, u, *ckpts)
        return u

    @staticmethod
    def backward(ctx, g):
        screens, final, *ckpts = ctx.saved_tensors
        dz, area, wl, every, K = ctx.geom
        g = g.contiguous().to(torch.complex64)
        need_phi = ctx.needs_input_grad[1]
        grad_screens = torch.empty_like(screens) if need_phi else None
        nseg = len(ckpts)
        for seg in reversed(range(nseg)):
            k0, k1 = seg * every, min(K, (seg + 1) * every)
            # Recompute u_{k0+1} .. u_{k1-1} from the checkpoint u_{k0}.
            states = [ckpts[seg]]
            for k in range(k0, k1 - 1):
                states.append(B.propagate_field(states[-1], area, wl, dz, xmask=screens[k],
                                                xmask_phase=True,
                                                flags=L.LP_FLAG_XMASK_AFTER))
            for k in reversed(range(k0, k1)):
                if need_phi:
                    y = states[k - k0 + 1] if k < k1 - 1 else (
                        ckpts[seg + 1] if seg + 1 < nseg else final)
                    B.phase_grad(y, g, out=grad_screens[k])     # Im(conj(y) * g)
                g = B.propagate_field(g, area, wl, dz, xmask=screens[k], xmask_phase=True,
                                      flags=L.LP_FLAG_ADJOINT | L.LP_FLAG_XMASK_AFTER)
            del states
        return g, grad_screens, None, None, None, None


def split_step_chain(field: torch.Tensor, screens: torch.Tensor, dz: float, area_size: float,
                     wl: float, checkpoint_every: int = 8) -> torch.Tensor:
    """K alternating steps of propagate(dz) and multiply by exp(i*screens[k]).

    screens: float32 (K, N, N).  Backward keeps ceil(K/checkpoint_every)
    fields and recomputes each segment, so peak memory is about
    (K/checkpoint_every + checkpoint_every) fields plus the screens.
    """
    if screens.dim() != 3 or screens.dtype != torch.float32:
        raise ValueError("screens must be a float32 (K, N, N) tensor")
    if checkpoint_every < 1:
        raise ValueError("checkpoint_every must be >= 1")
    return _Chain.apply(field.to(torch.complex64), screens.contiguous(), float(dz),
                        float(area_size), float(wl), int(checkpoint_every))
