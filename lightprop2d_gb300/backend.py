"""Tensor-level entry points over the C ABI (one call per C function).

Every function takes CUDA tensors (``torch.complex64`` grids of shape
``(N, N)``, row-major, unshifted spectra), launches on the current torch
stream of the tensor's device and returns without synchronising.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _grid(t: torch.Tensor, name: str, dtype=torch.complex64) -> int:
    if not isinstance(t, torch.Tensor):
        raise ValueError(f"{name} must be a torch tensor, got {type(t).__name__}")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if t.dim() != 2 or t.shape[0] != t.shape[1]:
        raise ValueError(f"{name} must be a square (N, N) grid, got {tuple(t.shape)}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t.shape[0]


_MASK_CODES = {
    torch.float32: L.LP_MASK_F32,
    torch.complex64: L.LP_MASK_C64,
    torch.bool: L.LP_MASK_U8,
    torch.uint8: L.LP_MASK_U8,
    torch.float64: L.LP_MASK_F64,
    torch.complex128: L.LP_MASK_C128,
}


def mask_arg(mask, n: int, device, name="mask", phase: bool = False):
    """(tensor, type-code) for an optional mask; numpy masks are uploaded.

    ``phase=True`` marks a float32 grid phi (radians) whose multiplier is
    exp(i*phi).  Returns (None, LP_MASK_NONE) for ``mask is None``.
    """
    if mask is None:
        return None, L.LP_MASK_NONE
    if hasattr(mask, "code") and hasattr(mask, "table"):  # generators.GenMask
        if mask.table.numel() != 2 * n or mask.table.device != torch.device(device):
            raise ValueError(f"{name}: compact generator table for a different grid")
        return mask.table, mask.code
    if isinstance(mask, np.ndarray):
        if mask.dtype == np.bool_:
            mask = torch.from_numpy(mask.astype(np.uint8))
        else:
            mask = torch.from_numpy(np.ascontiguousarray(mask))
    if not isinstance(mask, torch.Tensor):
        raise ValueError(f"{name} must be a numpy array or torch tensor")
    mask = mask.to(device=device)
    if mask.dtype == torch.bool:
        mask = mask.to(torch.uint8)
    if mask.dtype not in _MASK_CODES:
        mask = mask.to(torch.complex64 if mask.is_complex() else torch.float32)
    if tuple(mask.shape) != (n, n):
        mask = torch.broadcast_to(mask, (n, n))
    mask = mask.contiguous()
    code = _MASK_CODES[mask.dtype]
    if phase:
        if mask.dtype != torch.float32:
            mask = mask.to(torch.float32).contiguous()
        code = L.LP_MASK_PHASE_F32
    return mask, code


def _call(fn_name: str, dev, *args):
    lib = L.load()
    with torch.cuda.device(dev):
        st = _stream(dev)
        L.check(getattr(lib, fn_name)(*args, st), fn_name)


def init(device=None) -> None:
    if device is None:
        idx = torch.cuda.current_device()
    elif isinstance(device, int):
        idx = device
    else:
        idx = torch.device(device).index or 0
    L.check(L.load().lp_init(idx), "lp_init")


def is_supported(n: int) -> bool:
    return bool(L.load().lp_is_supported_n(int(n)))


def _zgrid(t: torch.Tensor, name: str):
    """(N, entry-point suffix) of a complex64 ("") or complex128 ("_c128") grid."""
    if isinstance(t, torch.Tensor) and t.dtype == torch.complex128:
        return _grid(t, name, torch.complex128), "_c128"
    return _grid(t, name), ""


def fft2(x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """numpy.fft.fft2 convention (beam2d.py:207-217); complex64 or complex128."""
    n, sfx = _zgrid(x, "x")
    out = torch.empty_like(x) if out is None else out
    _grid(out, "out", x.dtype)
    _call("lp_fft2" + sfx, x.device, _vp(x), _vp(out), n, 0)
    return out


def ifft2(x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """numpy.fft.ifft2 convention, 1/N^2 included (beam2d.py:219-229)."""
    n, sfx = _zgrid(x, "x")
    out = torch.empty_like(x) if out is None else out
    _grid(out, "out", x.dtype)
    _call("lp_fft2" + sfx, x.device, _vp(x), _vp(out), n, 1)
    return out


def propagate(spectrum: torch.Tensor, area_size: float, wl: float, z: float,
              field_out: torch.Tensor | None = None, kmask=None,
              write_spectrum: bool = True, flags: int = 0) -> torch.Tensor:
    """Beam2D.propagate (beam2d.py:481-490): spectrum *= kmask*H(z) (in place
    unless ``write_spectrum=False``) and return field = ifft2(spectrum)."""
    n, sfx = _zgrid(spectrum, "spectrum")
    field_out = torch.empty_like(spectrum) if field_out is None else field_out
    _grid(field_out, "field_out", spectrum.dtype)
    km, kc = mask_arg(kmask, n, spectrum.device, "kmask")
    if not write_spectrum:
        flags |= L.LP_FLAG_SPECTRUM_READONLY
    _call("lp_propagate" + sfx, spectrum.device, _vp(spectrum), _vp(field_out), n,
          float(area_size), float(wl), float(z), _vp(km), kc, int(flags))
    return field_out


def propagate_field(field: torch.Tensor, area_size: float, wl: float, z: float,
                    out: torch.Tensor | None = None, spectrum_out=None,
                    iprofile_out=None, lens_f: float = 0.0, xmask=None,
                    xmask_phase: bool = False, kmask=None, flags: int = 0) -> torch.Tensor:
    """Fused field -> field: [lens, xmask] -> fft2 -> [kmask] * H(z) -> ifft2.
    complex128 fields run the complex128 family (iprofile_out float64)."""
    n, sfx = _zgrid(field, "field")
    out = torch.empty_like(field) if out is None else out
    _grid(out, "out", field.dtype)
    if spectrum_out is not None:
        _grid(spectrum_out, "spectrum_out", field.dtype)
    if iprofile_out is not None:
        _grid(iprofile_out, "iprofile_out", torch.float64 if sfx else torch.float32)
    xm, xc = mask_arg(xmask, n, field.device, "xmask", phase=xmask_phase)
    km, kc = mask_arg(kmask, n, field.device, "kmask")
    _call("lp_propagate_field" + sfx, field.device, _vp(field), _vp(out), _vp(spectrum_out),
          _vp(iprofile_out), n, float(area_size), float(wl), float(z), float(lens_f),
          _vp(xm), xc, _vp(km), kc, int(flags))
    return out


def lens(field: torch.Tensor, area_size: float, wl: float, f: float,
         spectrum_out: torch.Tensor | None = None) -> None:
    """Beam2D.lens (beam2d.py:508-511) in place; optional spectrum = fft2(field)."""
    n, sfx = _zgrid(field, "field")
    if spectrum_out is not None:
        _grid(spectrum_out, "spectrum_out", field.dtype)
    _call("lp_lens" + sfx, field.device, _vp(field), _vp(spectrum_out), n, float(area_size),
          float(wl), float(f))


def coordinate_filter(field: torch.Tensor, mask, spectrum_out=None, phase=False) -> None:
    """Beam2D.coordinate_filter(f_init=mask) (beam2d.py:339-342) in place."""
    n, sfx = _zgrid(field, "field")
    if spectrum_out is not None:
        _grid(spectrum_out, "spectrum_out", field.dtype)
    m, c = mask_arg(mask, n, field.device, "mask", phase=phase)
    _call("lp_coordinate_filter" + sfx, field.device, _vp(field), _vp(spectrum_out), n, _vp(m), c)


def spectral_filter(spectrum: torch.Tensor, mask, field_out=None) -> torch.Tensor:
    """Beam2D.spectral_filter(f_init=mask) (beam2d.py:370-373)."""
    n, sfx = _zgrid(spectrum, "spectrum")
    field_out = torch.empty_like(spectrum) if field_out is None else field_out
    m, c = mask_arg(mask, n, spectrum.device, "mask")
    _call("lp_spectral_filter" + sfx, spectrum.device, _vp(spectrum), _vp(field_out), n, _vp(m), c)
    return field_out


def iprofile(field: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """|field|^2 as float32 (float64 for a complex128 field) (beam2d.py:717)."""
    n, sfx = _zgrid(field, "field")
    dt = torch.float64 if sfx else torch.float32
    out = torch.empty((n, n), dtype=dt, device=field.device) if out is None else out
    _grid(out, "out", dt)
    _call("lp_iprofile" + sfx, field.device, _vp(field), _vp(out), n)
    return out


def beam_moments(field: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Intensity moments (5 float64 on the device): sum I, sum jx I, sum jy I,
    sum (jx-xc)^2 I, sum (jy-yc)^2 I with grid-index offsets jx = ix - n/2
    (lp_beam_moments; Beam2D.centroid / D4sigma, beam2d.py:669-704)."""
    n = _grid(field, "field")
    out = torch.empty(5, dtype=torch.float64, device=field.device) if out is None else out
    if out.dtype != torch.float64 or out.numel() < 5 or not out.is_cuda:
        raise ValueError("out: float64 CUDA tensor of 5 elements")
    _call("lp_beam_moments", field.device, _vp(field), n, _vp(out))
    return out


def intensity_mse_sum(y: torch.Tensor, target: torch.Tensor,
                      out: torch.Tensor | None = None) -> torch.Tensor:
    """sum (|y|^2 - target)^2 as one float64 on the device (lp_intensity_mse)."""
    _check_loss_args(y, target)
    out = torch.empty(1, dtype=torch.float64, device=y.device) if out is None else out
    _call("lp_intensity_mse", y.device, _vp(y), _vp(target), y.numel(), _vp(out))
    return out


def intensity_mse_grad(y: torch.Tensor, target: torch.Tensor, upstream: torch.Tensor,
                       scale: float, out: torch.Tensor | None = None) -> torch.Tensor:
    """upstream * scale * (|y|^2 - target) * y (lp_intensity_mse_grad); upstream
    is a one-element float32 CUDA tensor read on the device."""
    _check_loss_args(y, target)
    if upstream.dtype != torch.float32 or not upstream.is_cuda or upstream.numel() != 1:
        raise ValueError("upstream: one-element float32 CUDA tensor")
    out = torch.empty_like(y) if out is None else out
    _call("lp_intensity_mse_grad", y.device, _vp(y), _vp(target), y.numel(),
          _vp(upstream.contiguous()), float(scale), _vp(out))
    return out


def phase_grad(x: torch.Tensor, g: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Im(conj(x) * g) as float32 (lp_phase_grad): the gradient of a real loss
    with respect to a phase mask applied as x = u * exp(i*phi)."""
    for t, nm in ((x, "x"), (g, "g")):
        if t.dtype != torch.complex64 or not t.is_cuda or not t.is_contiguous():
            raise ValueError(f"{nm}: contiguous complex64 CUDA tensor")
    if g.shape != x.shape:
        raise ValueError("g must have x's shape")
    out = torch.empty(x.shape, dtype=torch.float32, device=x.device) if out is None else out
    _call("lp_phase_grad", x.device, _vp(x), _vp(g), x.numel(), _vp(out))
    return out


def _check_loss_args(y: torch.Tensor, target: torch.Tensor) -> None:
    if y.dtype != torch.complex64 or not y.is_cuda or not y.is_contiguous():
        raise ValueError("y: contiguous complex64 CUDA tensor")
    if target.dtype != torch.float32 or target.shape != y.shape or not target.is_contiguous():
        raise ValueError("target: contiguous float32 tensor of y's shape")


def expand(field: torch.Tensor, n_out: int) -> torch.Tensor:
    """Edge-replicated padding to n_out x n_out (lp_expand; beam2d.py:375-404)."""
    n = _grid(field, "field")
    out = torch.empty((n_out, n_out), dtype=torch.complex64, device=field.device)
    _call("lp_expand", field.device, _vp(field), n, _vp(out), int(n_out))
    return out


def coarse(field: torch.Tensor, order: int) -> torch.Tensor:
    """order x order block mean (lp_coarse; beam2d.py:434-460)."""
    n = _grid(field, "field")
    if order < 1 or n % order:
        raise ValueError(f"mean_order={order} must divide npoints={n}")
    out = torch.empty((n // order, n // order), dtype=torch.complex64, device=field.device)
    _call("lp_coarse", field.device, _vp(field), n, _vp(out), int(order))
    return out


def crop(field: torch.Tensor, first: int, n_keep: int, x0: float, dL_in: float, n_out: int,
         dL_out: float) -> torch.Tensor:
    """Bilinear resampling of the window field[first:first+n_keep]^2 onto the
    centred n_out grid of spacing dL_out (lp_crop; beam2d.py:406-432)."""
    n = _grid(field, "field")
    out = torch.empty((n_out, n_out), dtype=torch.complex64, device=field.device)
    _call("lp_crop", field.device, _vp(field), n, int(first), int(n_keep), float(x0),
          float(dL_in), _vp(out), int(n_out), float(dL_out))
    return out


def apply_transfer(spectrum: torch.Tensor, area_size: float, wl: float, z: float,
                   flags: int = 0) -> None:
    """spectrum *= H(z) in place."""
    n, sfx = _zgrid(spectrum, "spectrum")
    _call("lp_apply_transfer" + sfx, spectrum.device, _vp(spectrum), n, float(area_size),
          float(wl), float(z), int(flags))


def plain_propagate_field(field: torch.Tensor, area_size: float, wl: float, z: float,
                          out: torch.Tensor | None = None, fp64_h: bool = False,
                          flags: int = 0) -> torch.Tensor:
    """Unfused comparison form: fft2, H grid in HBM, multiply, ifft2."""
    n = _grid(field, "field")
    out = torch.empty_like(field) if out is None else out
    if fp64_h:
        flags |= L.LP_FLAG_PLAIN_FP64_H
    _call("lp_plain_propagate_field", field.device, _vp(field), _vp(out), n,
          float(area_size), float(wl), float(z), int(flags))
    return out
