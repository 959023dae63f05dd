"""``Beam2D`` with the API of lightprop2d/beam2d.py, backed by GB300 CUDA kernels.

Same dataclass fields, methods and results as the reference class
(beam2d.py:44-757) for the propagation path: the constructor, ``propagate``,
``lens``, ``coordinate_filter``, ``spectral_filter``, ``field``,
``spectrum``, ``iprofile``, ``phiprofile`` and the grid attributes
``X, Y, Kx, Ky, Kz, k0, dL``.

How the state is kept (observable results are the reference's):

* ``field`` is a CUDA tensor of ``complex`` (complex128 for
  ``complex_bits=128``, the reference's default, else complex64).  Each operation that
  replaces the field allocates a new tensor, as the reference rebinds
  ``self.field``.
* The spectrum is state (beam2d.py:489).  It is stored as a base grid plus a
  pending propagation distance ``dz``: ``spectrum = base * H(dz)``.  So a
  run of ``propagate`` calls reads the base spectrum and writes the field
  (one inverse 2-D FFT per call, ``H`` made in registers), and the spectrum
  is only multiplied out when someone reads ``beam.spectrum``.
* After ``lens`` / ``coordinate_filter`` the reference recomputes
  ``spectrum = fft2(field)``.  Here the x-domain multiplier is kept pending
  and folded into the next transform, so ``lens(f); propagate(z)`` is one
  fused field -> field pass sequence (lens in the first pass, H between the
  forward and inverse column transforms).
* Grids ``X, Y, Kx, Ky`` are host numpy arrays like the reference's CPU
  path, so generator callables (``init_field_gen``, ``f_gen``) receive the
  same arguments as in the reference; their results are uploaded once.

Differences, by design:

* ``complex_bits=128`` runs the propagation path (transforms, propagate,
  lens, filters, iprofile) in the FP64 kernel family and agrees with the
  reference's complex128 path to round-off; ``complex_bits=64`` runs the
  fused complex64 kernels (FP64-grade transfer phases, ~1e-7 relative L2).
  Beam metrics, grid management and mode decomposition compute in complex64
  for either (results cast back to the beam's dtype).
* ``use_gpu`` is accepted for signature compatibility; the backend always
  runs on a CUDA device.  ``numpy_output`` works as in the reference.
* Supported ``npoints``: any from 2 to 4096, and powers of two up to 8192
  (ValueError otherwise).
"""
from __future__ import annotations

import math
from collections.abc import Iterable
from dataclasses import dataclass
from typing import Callable, Union

import numpy as np
import torch

from . import backend as B
from . import generators as G
from . import modes as M

nm = 1e-7
um = 1e-4
mm = 1e-1
cm = 1
m = 100



def _to_device(a, device, dtype=torch.complex64) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        t = a.to(device=device)
    elif isinstance(a, np.ndarray) or np.isscalar(a):
        t = torch.as_tensor(np.ascontiguousarray(a), device=device)
    else:
        raise ValueError("Unknown type of the given array, not numpy array or torch tensor")
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    return t.contiguous()


@dataclass
class Beam2D:
    """Electromagnetic field propagation using the spectral (angular-spectrum) method.

    Parameters are those of lightprop2d.Beam2D (beam2d.py:79-91), lengths in cm.
    """

    area_size: float
    npoints: int
    wl: float
    z: float = 0.
    xp: object = torch
    init_field: object = None
    init_spectrum: object = None
    init_field_gen: object = None
    init_gen_args: tuple = ()
    complex_bits: int = 128

    use_gpu: bool = False
    numpy_output: bool = True
    device: object = None

    # ------------------------------------------------------------ set-up --
    def __post_init__(self):
        self.xp = torch
        if self.device is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(self.device)
        if self.device.type != "cuda":
            raise ValueError("the GB300 backend needs a CUDA device")
        if not B.is_supported(self.npoints):
            raise ValueError(
                f"npoints={self.npoints} is not supported by the GB300 backend "
                "(powers of two from 16 to 8192)")
        if self.complex_bits == 64:
            self.complex = torch.complex64
        elif self.complex_bits == 128:
            self.complex = torch.complex128
        else:
            raise ValueError("complex_bits must be 64 or 128")
        B.init(self.device)
        self._construct_grids()
        if self.init_field_gen is not None:
            f = self.init_field_gen(self.X, self.Y, *self.init_gen_args)
        elif self.init_field is not None:
            f = self.init_field
        else:
            raise ValueError(
                "Init field data is None : " +
                "'init_field_gen' must be a function or 'init_field' must be an array.")
        self._field = _to_device(f, self.device, self.complex)
        self._check_grid(self._field, "init field")
        self._pend_invf = 0.0   # pending lens: sum of 1/f
        self._pend_xmask = None  # pending coordinate mask (device tensor)
        if self.init_spectrum is None:
            self._spec = None    # derived: fft2(field)
        else:
            self._spec = _to_device(self.init_spectrum, self.device, self.complex)
            self._check_grid(self._spec, "init spectrum")
        self._spec_dz = 0.0

    def _check_grid(self, t, what):
        if tuple(t.shape) != (self.npoints, self.npoints):
            raise ValueError(f"{what} must be {self.npoints}x{self.npoints}, "
                             f"got {tuple(t.shape)}")

    def _construct_grids(self):
        """Grids as in beam2d.py:299-308; Kz is computed lazily on access."""
        self.dL = self.area_size / self.npoints
        self.X = np.arange(-self.npoints // 2, self.npoints // 2, 1) * self.dL
        self.Y = self.X.reshape((-1, 1))
        self._X0 = self.X.copy()  # to detect in-place changes of X (see lens)
        self.k0 = 1 / self.wl
        self.Kx = np.fft.fftfreq(self.npoints, d=self.dL)
        self.Ky = self.Kx.reshape((-1, 1))
        self._Kz = None
        self._xscale = 1.0  # factor lens_image leaves on X (beam2d.py:529-531)

    @property
    def Kz(self):
        if self._Kz is None:
            with np.errstate(invalid="ignore"):
                self._Kz = np.nan_to_num(np.sqrt(self.k0 ** 2 - self.Kx ** 2 - self.Ky ** 2))
        return self._Kz

    # -------------------------------------------------------------- state --
    def _c64(self, t):
        """The complex64 view that the metrics, grid and mode kernels take."""
        return t if t.dtype == torch.complex64 else t.to(torch.complex64)

    def _has_pending(self) -> bool:
        return self._pend_invf != 0.0 or self._pend_xmask is not None

    def _flush_x(self):
        """Apply pending x-domain multipliers to the field (new tensor)."""
        if not self._has_pending():
            return
        f = self._field.clone()
        if self._pend_invf != 0.0:
            B.lens(f, self.area_size, self.wl, 1.0 / self._pend_invf)
        if self._pend_xmask is not None:
            B.coordinate_filter(f, self._pend_xmask)
        self._field = f
        self._pend_invf = 0.0
        self._pend_xmask = None

    @property
    def field(self) -> torch.Tensor:
        self._flush_x()
        return self._field

    @field.setter
    def field(self, value):
        # The reference keeps the spectrum when the field is assigned directly.
        if self._spec is None:
            self._materialise_spectrum()
        self._pend_invf = 0.0
        self._pend_xmask = None
        self._field = _to_device(value, self.device, self.complex)
        self._check_grid(self._field, "field")

    def _materialise_spectrum(self):
        if self._spec is None:
            self._flush_x()
            self._spec = B.fft2(self._field)
            self._spec_dz = 0.0
        elif self._spec_dz != 0.0:
            s = self._spec.clone()
            B.apply_transfer(s, self.area_size, self.wl, self._spec_dz)
            self._spec = s
            self._spec_dz = 0.0

    @property
    def spectrum(self) -> torch.Tensor:
        self._materialise_spectrum()
        return self._spec

    @spectrum.setter
    def spectrum(self, value):
        self._spec = _to_device(value, self.device, self.complex)
        self._check_grid(self._spec, "spectrum")
        self._spec_dz = 0.0

    # ---------------------------------------------------------- operators --
    def _update_obj(self, field, spectrum=None):
        """beam2d.py:231-288: reset z and swap in a new field (and spectrum)."""
        self.z = 0
        self._pend_invf = 0.0
        self._pend_xmask = None
        self._field = _to_device(field, self.device, self.complex)
        self._spec = None if spectrum is None else _to_device(spectrum, self.device, self.complex)
        self._spec_dz = 0.0

    def propagate(self, z: float):
        """Propagate by ``z`` cm (beam2d.py:462-490).

        spectrum *= exp(-2*pi*i*Kz*z); field = ifft2(spectrum).
        """
        if z == 0:
            return
        self.z += z
        if self._spec is not None:
            # Spectrum is state: read base spectrum, apply H(dz_total) in
            # registers, write only the field.
            self._spec_dz += z
            self._field = B.propagate(self._spec, self.area_size, self.wl, self._spec_dz,
                                      write_spectrum=False)
            return
        # Spectrum derived from the field (+ pending lens/mask): one fused
        # field -> field sequence that also stores the propagated spectrum.
        spec = torch.empty_like(self._field)
        lens_f = (1.0 / self._pend_invf) if self._pend_invf != 0.0 else 0.0
        self._field = B.propagate_field(self._field, self.area_size, self.wl, z,
                                        spectrum_out=spec, lens_f=lens_f,
                                        xmask=self._pend_xmask)
        self._pend_invf = 0.0
        self._pend_xmask = None
        self._spec = spec
        self._spec_dz = 0.0

    def lens(self, f: float):
        """Thin lens exp(i*(X^2+Y^2)*k0/(2f)) (beam2d.py:492-511)."""
        if not (isinstance(f, (int, float, np.floating)) and math.isfinite(f) and f != 0):
            raise ValueError("focal length must be a finite non-zero number")
        if not np.array_equal(self.X, self._X0 * self._xscale):
            # The reference builds the phase from self.X, which profile
            # generators shift in place (gaussian_beam's `x -= x0` on the grid
            # and its Y view): centre the lens there, in FP64 on the device.
            X = torch.as_tensor(self.X, dtype=torch.float64, device=self.device)
            ph = torch.remainder((X[None, :] ** 2 + X[:, None] ** 2) * (self.k0 / (2 * f)),
                                 2 * math.pi)
            self.coordinate_filter(f_init=torch.polar(torch.ones_like(ph), ph).to(self.complex))
            return
        self._pend_invf += self._xscale ** 2 / f  # the phase follows the (scaled) grid X
        self._spec = None
        self._spec_dz = 0.0

    def _mask(self, f_init, f_gen, fargs, grid_x, grid_y):
        m = None
        if f_gen is not None:
            assert callable(f_gen)
            assert isinstance(fargs, Iterable)
            m = _to_device(f_gen(grid_x, grid_y, *fargs), self.device, dtype=None)
        if f_init is not None:
            assert isinstance(f_init, (np.ndarray, torch.Tensor))
            fi = _to_device(f_init, self.device, dtype=None)
            m = fi if m is None else m * fi
        if m is not None and m.dtype == torch.bool:
            m = m.to(torch.uint8)
        return m

    def coordinate_filter(self, f_init=None, f_gen: Union[Callable, None] = None,
                          fargs: tuple = ()) -> None:
        """field *= f_gen(X, Y, *fargs) * f_init; spectrum = fft2(field)
        (beam2d.py:310-342)."""
        m = None
        if f_init is None and f_gen is not None and self.complex == torch.complex64:
            # deterministic generators become a 2N table evaluated in the pass
            # (complex128 beams keep the generator's float64 mask)
            m = G.compact(f_gen, fargs, self.X, self.Y, self.device)
        if m is None:
            m = self._mask(f_init, f_gen, fargs, self.X, self.Y)
        if m is None:
            self._flush_x()
            self._spec = None
            return
        if self._pend_xmask is not None:
            self._flush_x()
        self._pend_xmask = m
        self._spec = None
        self._spec_dz = 0.0

    def spectral_filter(self, f_init=None, f_gen: Union[Callable, None] = None,
                        fargs: tuple = ()) -> None:
        """spectrum *= f_gen(Kx, Ky, *fargs) * f_init; field = ifft2(spectrum)
        (beam2d.py:344-373)."""
        m = None
        if f_init is None and f_gen is not None and self.complex == torch.complex64:
            m = G.compact(f_gen, fargs, self.Kx, self.Ky, self.device, allow_span=False)
        if m is None:
            m = self._mask(f_init, f_gen, fargs, self.Kx, self.Ky)
        if self._spec is None:
            spec = torch.empty_like(self._field)
            lens_f = (1.0 / self._pend_invf) if self._pend_invf != 0.0 else 0.0
            self._field = B.propagate_field(self._field, self.area_size, self.wl, 0.0,
                                            spectrum_out=spec, lens_f=lens_f,
                                            xmask=self._pend_xmask, kmask=m)
            self._pend_invf = 0.0
            self._pend_xmask = None
            self._spec = spec
        else:
            spec = self._spec.clone()
            self._field = B.propagate(spec, self.area_size, self.wl, self._spec_dz, kmask=m)
            self._spec = spec
        self._spec_dz = 0.0

    # ----------------------------------------------------------- readouts --
    def _np(self, t):
        """A numpy copy of t when numpy_output (a new array per call, as the
        reference returns), else t.  The copy lands in page-locked memory from
        torch's host allocator cache, so it runs at the host link's DMA rate
        and a read-back loop reuses the blocks of the arrays it dropped."""
        if not self.numpy_output:
            return t
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        return h.numpy()

    @property
    def iprofile(self):
        """|field|^2 (beam2d.py:706-721); numpy when numpy_output."""
        return self._np(B.iprofile(self.field))

    @property
    def phiprofile(self):
        """angle(field) (beam2d.py:723-738); numpy when numpy_output."""
        return self._np(torch.angle(self.field))

    def _moments(self):
        """(m0, m1, m2, m3, m4) of lp_beam_moments on the host; the reference's
        np.average raises ZeroDivisionError for a zero field, so does this."""
        m = B.beam_moments(self._c64(self.field)).cpu().tolist()
        if not m[0] > 0:
            raise ZeroDivisionError("Weights sum to zero, can't be normalized")
        return m

    @property
    def centroid(self):
        """Intensity-weighted centre (Xc, Yc, nxc, nyc) (beam2d.py:669-685)."""
        n = self.npoints // 2
        m = self._moments()
        Xc = self.dL * (m[1] / m[0])
        Yc = self.dL * (m[2] / m[0])
        return Xc, Yc, int(Xc / self.dL) + n, int(Yc / self.dL) + n

    @property
    def D4sigma(self):
        """Beam widths 4*sigma along x and y (beam2d.py:687-704)."""
        m = self._moments()
        return 4 * self.dL * math.sqrt(m[3] / m[0]), 4 * self.dL * math.sqrt(m[4] / m[0])

    @property
    def centroid_intensity(self) -> float:
        """Intensity at the centroid pixel (beam2d.py:740-752)."""
        _, _, nxc, nyc = self.centroid
        v = self.field[nyc, nxc]
        return float(v.real ** 2 + v.imag ** 2)

    # --------------------------------------------------- grid management --
    def _regrid(self, field):
        """Swap in a field on the new grid; the spectrum is fft2(field), made
        when read (the reference computes it eagerly)."""
        self._field = field.to(self.complex)
        self._pend_invf = 0.0
        self._pend_xmask = None
        self._spec = None
        self._spec_dz = 0.0

    def _check_new_n(self, n, what):
        if not B.is_supported(n):
            raise ValueError(f"{what}: npoints={n} is not supported by the GB300 backend "
                             "(powers of two from 16 to 8192)")

    def expand(self, area_size: float):
        """Grow the area to ``area_size`` at constant dL, padding every side
        with copies of the edge values (beam2d.py:375-404)."""
        old = self.npoints
        n = int(self.npoints * area_size / self.area_size)
        n -= n % 2
        if n < old:
            raise ValueError("expand: the new area must not be smaller than the current one")
        self._check_new_n(n, "expand")
        f = B.expand(self._c64(self.field), n)
        self.npoints = n
        self.area_size = area_size
        self._construct_grids()
        self._regrid(f)

    def crop(self, area_size: float, npoints: int = 0):
        """Resample the central window |X| < area_size/2 onto a grid of
        ``area_size`` and ``npoints`` points (the current count if 0) by
        bilinear interpolation, as the reference's ``interp2d`` does
        (beam2d.py:406-432)."""
        nc = self.npoints // 2
        n = int(np.count_nonzero(np.abs(self.X) < area_size / 2)) // 2
        if n < 1:
            raise ValueError("crop: the window holds no grid points")
        first = nc - n
        x0, dL_in = float(self.X[first]), self.dL
        new_n = npoints if npoints else self.npoints
        self._check_new_n(new_n, "crop")
        f = self._c64(self.field)
        self.npoints = new_n
        self.area_size = area_size
        self._construct_grids()
        self._regrid(B.crop(f, first, 2 * n, x0, dL_in, new_n, self.dL))

    def coarse(self, mean_order: int = 1):
        """Divide npoints by ``mean_order`` with a block mean of the field
        (beam2d.py:434-460)."""
        if mean_order < 1 or self.npoints % mean_order:
            raise ValueError(f"coarse: mean_order={mean_order} must divide npoints={self.npoints}")
        n = self.npoints // mean_order
        self._check_new_n(n, "coarse")
        f = B.coarse(self._c64(self.field), mean_order)
        self.npoints = n
        self._construct_grids()
        self._regrid(f)

    # ---------------------------------------------- outside this backend --
    def lens_image(self, f: float, l1: float, l2: float):
        """Image through a lens between conjugate planes (beam2d.py:513-537):
        field = s * field(s*X, s*Y) * exp(-i*(X^2+Y^2)*k0*(l1+l2)/(2*l2^2)),
        s = -l1/l2, resampled bilinearly like the reference's interp2d.  As
        there, the sample coordinates are sorted before evaluation (so a
        negative s does not mirror the image), and the grid X (and its view
        Y) is left scaled by s; later lenses follow that scaled grid."""
        if not (l2 != 0 and math.isfinite(l1) and math.isfinite(l2)):
            raise ValueError("lens_image: l1, l2 finite and l2 non-zero")
        if self._xscale < 0:
            raise NotImplementedError("lens_image on a grid mirrored by a previous lens_image")
        s = -l1 / l2
        if s == 0:
            raise ValueError("lens_image: l1 must be non-zero")
        n = self.npoints
        dL_in = float(self.X[1] - self.X[0])
        x0 = float(self.X[0]) - (abs(s) * dL_in if s < 0 else 0.0)
        g = B.crop(self._c64(self.field), 0, n, x0, dL_in, n, abs(s) * dL_in)
        g *= s
        self._regrid(g)
        # phase = -(X^2+Y^2)*k0*(l1+l2)/(2*l2^2): a lens of focal length
        # -l2^2/(l1+l2) on the current grid
        if l1 + l2 != 0:
            self.lens(-l2 ** 2 / (l1 + l2))
        self.X *= s
        self._xscale *= s

    # ------------------------------------------------- mode decomposition --
    def _coeffs_out(self, c: torch.Tensor):
        self.modes_coeffs = c.cpu().numpy() if self.numpy_output else c
        return self.modes_coeffs

    def deconstruct_by_modes(self, modes_list, mode: str = "scalar"):
        """Mode coefficients of the central window of the field
        (beam2d.py:561-600): ``scalar`` = modes @ window (lp_modes_project),
        ``lstsq`` = least-squares solution.  ``modes_list`` may be a
        ``ModeBasis`` (uploaded once) or a list / array of flattened modes."""
        basis = M.ModeBasis(modes_list, self.device)
        if mode == "scalar":
            c = M.project(basis, self._c64(self.field))
        elif mode == "lstsq":
            c = M.lstsq(basis, self._c64(self.field))
        else:
            raise ValueError(f"unknown mode {mode!r}: 'scalar' or 'lstsq'")
        return self._coeffs_out(c)

    def fast_deconstruct_by_modes(self, modes_matrix_t, modes_matrix_dot_t):
        """lstsq(modes_matrix_dot_t, modes_matrix_t . window) (beam2d.py:602-648)."""
        return self._coeffs_out(M.fast_lstsq(modes_matrix_t, modes_matrix_dot_t,
                                             self._c64(self.field)))

    def construct_by_modes(self, modes_list, modes_coeffs):
        """field = sum_i c_i * mode_i, zero outside the modes' window; the
        spectrum follows (beam2d.py:650-667)."""
        basis = M.ModeBasis(modes_list, self.device)
        self._regrid(M.combine(basis, modes_coeffs, self.npoints, self.device))

    def __repr__(self) -> str:
        return (f"Beam {self.npoints:d}x{self.npoints:d} points" +
                f"\n\t{self.area_size:.3g}x{self.area_size:.3g} cm " +
                f"\n\t<wl={self.wl / nm:.3g} nm, z={self.z:.3g} cm>")
