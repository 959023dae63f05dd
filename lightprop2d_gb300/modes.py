"""Mode decomposition on the device (Beam2D.deconstruct_by_modes,
fast_deconstruct_by_modes, construct_by_modes; beam2d.py:539-667).

``ModeBasis`` uploads a mode list once (complex64, n_modes x nb^2) so a loop of
decompositions reads it from HBM only.  The projection and the synthesis are
the library's own kernels (``lp_modes_project`` / ``lp_modes_combine``); the
least-squares variants solve the small normal system with torch.linalg
(cuSOLVER) in complex128 after the large products ran in those kernels.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L


class ModeBasis:
    """Modes as rows of an (n_modes, nb*nb) complex64 device matrix."""

    def __init__(self, modes_list, device=None):
        device = (torch.device(device) if device is not None
                  else torch.device("cuda", torch.cuda.current_device()))
        if isinstance(modes_list, ModeBasis):
            self.matrix, self.nb = modes_list.matrix, modes_list.nb
            return
        if isinstance(modes_list, torch.Tensor):
            m = modes_list.to(device=device, dtype=torch.complex64)
        else:
            m = torch.as_tensor(np.ascontiguousarray(np.asarray(modes_list)), device=device)
            m = m.to(torch.complex64)
        if m.dim() != 2:
            m = m.reshape(m.shape[0], -1)
        nb = int(round(np.sqrt(m.shape[1])))
        if nb * nb != m.shape[1]:
            raise ValueError("modes must be flattened square grids (nb*nb points each)")
        self.matrix = m.contiguous()
        self.nb = nb

    @property
    def n_modes(self) -> int:
        return self.matrix.shape[0]


def _call(fn, dev, *args):
    lib = L.load()
    with torch.cuda.device(dev):
        st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        L.check(getattr(lib, fn)(*args, st), fn)


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def project(basis: ModeBasis, field: torch.Tensor) -> torch.Tensor:
    """complex128 (n_modes,) = modes @ window(field) (beam2d.py:593-596)."""
    n = field.shape[0]
    if basis.nb > n or (n - basis.nb) % 2:
        raise ValueError(f"mode grid {basis.nb} does not fit the field grid {n}")
    c = torch.empty(basis.n_modes, dtype=torch.complex128, device=field.device)
    _call("lp_modes_project", field.device, _vp(basis.matrix), basis.n_modes, basis.nb,
          _vp(field), n, _vp(c))
    return c


def combine(basis: ModeBasis, coeffs, n: int, device) -> torch.Tensor:
    """n x n complex64 field = sum_m coeffs[m] * mode_m, zero outside the
    central window (beam2d.py:539-559, :650-667)."""
    if basis.nb > n or (n - basis.nb) % 2:
        raise ValueError(f"mode grid {basis.nb} does not fit the field grid {n}")
    c = torch.as_tensor(np.asarray(coeffs) if not isinstance(coeffs, torch.Tensor) else coeffs,
                        device=device).to(torch.complex128).contiguous()
    if c.numel() != basis.n_modes:
        raise ValueError(f"{c.numel()} coefficients for {basis.n_modes} modes")
    out = torch.empty((n, n), dtype=torch.complex64, device=device)
    _call("lp_modes_combine", device, _vp(basis.matrix), basis.n_modes, basis.nb, _vp(c),
          _vp(out), n)
    return out


def lstsq(basis: ModeBasis, field: torch.Tensor) -> torch.Tensor:
    """argmin_c ||modes^T c - window|| (mode="lstsq", beam2d.py:597-599):
    normal equations (A^H A) c = A^H w with A = modes^T, in complex128."""
    n = field.shape[0]
    f0 = (n - basis.nb) // 2
    w = field[f0:f0 + basis.nb, f0:f0 + basis.nb].reshape(-1).to(torch.complex128)
    A = basis.matrix.to(torch.complex128)          # (M, P) = (modes^T)^T
    G = torch.conj(A) @ A.transpose(0, 1)            # A^H A with A = modes^T: (M, M)
    rhs = torch.conj(A) @ w
    return torch.linalg.solve(G, rhs)


def fast_lstsq(modes_matrix_t, modes_matrix_dot_t, field: torch.Tensor) -> torch.Tensor:
    """fast_deconstruct_by_modes (beam2d.py:602-648): lstsq(G, M_t . window)."""
    basis = ModeBasis(modes_matrix_t, field.device)
    rhs = project(basis, field)
    G = torch.as_tensor(np.asarray(modes_matrix_dot_t) if not isinstance(modes_matrix_dot_t,
                                                                         torch.Tensor)
                        else modes_matrix_dot_t, device=field.device).to(torch.complex128)
    return torch.linalg.lstsq(G, rhs.unsqueeze(1)).solution.squeeze(1)
