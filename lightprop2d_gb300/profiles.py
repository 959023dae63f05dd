"""Initial-field and mask generators with the semantics of lightprop2d/profiles.py.

Each generator takes the Beam2D grids ``x`` (1-D row, length N) and ``y``
(column, N x 1) and returns an N x N array.  numpy inputs give numpy outputs
(this is what ``Beam2D`` passes, like the reference); torch inputs give
tensors on the same device.

Reference behaviours kept on purpose, because a drop-in must reproduce them:

* ``gaussian_beam`` shifts its ``x``/``y`` arguments in place by ``x0``/``y0``
  (profiles.py:69-70).
* ``round_hole`` thresholds a Gaussian of width R at exp(-1/2), so the hole's
  geometric radius is R/sqrt(2) (profiles.py:79-80).
* the random generators draw from the global RNG of the array library
  (numpy.random / torch's default generator), profiles.py:45-61.
"""
from __future__ import annotations

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is a hard dependency of the package
    torch = None

__all__ = ('plane_wave', 'random_wave', 'random_wave_bin', 'gaussian_beam',
           'round_hole', 'random_round_hole', 'random_round_hole_bin',
           'random_round_hole_phase', 'rectangle_hole', 'square_hole',
           'square_slits')


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


def _shape(x, y):
    return (len(y), len(x)) if not _is_torch(x) else (y.shape[0], x.shape[-1])


def binning(field, binning_order: int):
    """Kronecker upsampling by a block of ones (profiles.py:29-32)."""
    if _is_torch(field):
        ones = torch.ones((binning_order, binning_order), dtype=field.dtype,
                          device=field.device)
        return torch.kron(field, ones)
    return np.kron(field, np.ones((binning_order, binning_order)))


def plane_wave(x, y):
    """All-ones grid (profiles.py:35-38)."""
    if _is_torch(x):
        return torch.ones(_shape(x, y), dtype=torch.float64, device=x.device)
    return np.ones(_shape(x, y))


def _uniform(shape, like):
    if _is_torch(like):
        return torch.rand(shape, dtype=torch.float64, device=like.device)
    return np.random.uniform(size=shape)


def _randint01(shape, like):
    if _is_torch(like):
        return torch.randint(0, 2, shape, device=like.device)
    return np.random.randint(0, 2, size=shape)


def random_wave_bin(x, y, binning_order: int = 1):
    """Binary random grid on blocks of binning_order^2 (profiles.py:41-50)."""
    ny, nx = _shape(x, y)
    return binning(_randint01((int(ny // binning_order), int(nx // binning_order)), x),
                   binning_order)


def random_wave(x, y, binning_order: int = 1):
    """Uniform [0,1) random grid on blocks of binning_order^2 (profiles.py:53-61)."""
    ny, nx = _shape(x, y)
    return binning(_uniform((int(ny // binning_order), int(nx // binning_order)), x),
                   binning_order)


def gaussian_beam(x, y, A0: float, rho0: float, x0: float = 0, y0: float = 0):
    """A0*exp(-((x-x0)^2+(y-y0)^2)/rho0^2); shifts x, y in place (profiles.py:64-71)."""
    x -= x0
    y -= y0
    if _is_torch(x):
        return A0 * torch.exp(-(x ** 2 + y ** 2) / rho0 ** 2)
    return A0 * np.exp(-(x ** 2 + y ** 2) / rho0 ** 2)


def round_hole(x, y, R: float, x0: float = 0, y0: float = 0):
    """Boolean disc exp(-r^2/R^2) >= exp(-1/2), radius R/sqrt(2) (profiles.py:74-81)."""
    d = gaussian_beam(x - x0, y - y0, 1, R)
    thr = 1 / np.exp(0.5)
    return d >= thr


def random_round_hole_bin(x, y, R: float, x0: float = 0, y0: float = 0,
                          binning_order: int = 1):
    """random_wave_bin zeroed outside round_hole (profiles.py:84-91)."""
    field = random_wave_bin(x, y, binning_order)
    field[round_hole(x, y, R, x0, y0) == 0] = 0
    return field


def random_round_hole(x, y, R: float, x0: float = 0, y0: float = 0,
                      binning_order: int = 1):
    """random_wave zeroed outside round_hole (profiles.py:94-101)."""
    field = random_wave(x, y, binning_order)
    field[round_hole(x, y, R, x0, y0) == 0] = 0
    return field


def random_round_hole_phase(x, y, R: float, x0: float = 0, y0: float = 0,
                            binning_order: int = 1):
    """Unit-amplitude random phase 2*pi*U inside round_hole (profiles.py:104-113)."""
    angle = random_round_hole(x, y, R, x0, y0, binning_order) * 2 * np.pi
    if _is_torch(angle):
        phase = torch.cos(angle) + 1j * torch.sin(angle)
    else:
        phase = np.cos(angle) + 1j * np.sin(angle)
    return round_hole(x, y, R, x0, y0) * phase


def rectangle_hole(x, y, dx: float, dy: float, x0=0, y0=0):
    """|x-x0| < dx/2 and |y-y0| < dy/2 (profiles.py:116-121)."""
    if _is_torch(x):
        return (torch.abs(x - x0) < (dx / 2)) & (torch.abs(y - y0) < (dy / 2))
    return (np.abs(x - x0) < (dx / 2)) & (np.abs(y - y0) < (dy / 2))


def square_hole(x, y, d: float, x0: float = 0, y0: float = 0):
    """rectangle_hole with dx = dy = d (profiles.py:124-128)."""
    return rectangle_hole(x, y, d, d, x0, y0)


def square_slits(x, y, d: float, slits_distance: float, x0: float = 0, y0: float = 0):
    """Two square holes at x0 -+ slits_distance/2 (profiles.py:131-136)."""
    dl = slits_distance / 2
    return square_hole(x, y, d, x0 - dl, y0) | square_hole(x, y, d, x0 + dl, y0)
