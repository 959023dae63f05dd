"""Compact device-side forms of the profile generators used as masks.

``Beam2D.coordinate_filter(f_gen=round_hole, fargs=(R,))`` and friends
(beam2d.py:310-342 with the generators of profiles.py:64-136) would build an
N x N mask on the host.  The deterministic generators are separable or
row-interval shaped, so here they become 2*N-entry tables that the first
FFT pass evaluates per point (mask types LP_MASK_SEP_F32 / LP_MASK_SPAN_I32):

* ``gaussian_beam``   fx[ix] * fy[iy], fx = A0*exp(-x^2/rho0^2), fy = exp(-y^2/rho0^2)
* ``rectangle_hole``, ``square_hole``, ``square_slits``, ``plane_wave``
                      0/1 (or 1) per axis, product
* ``round_hole``      rows lo[ix] <= iy < hi[ix] per column

Each table entry is computed with the reference's own float64 expressions on
the same coordinate arrays, so boolean edges are the reference's edges
exactly (the round-hole spans are found by evaluating its exact
``exp(-(x^2+y^2)/R^2) >= 1/exp(0.5)`` test in a window around the analytic
boundary).  ``gaussian_beam`` shifts the caller's coordinate arrays in place,
as the reference does (``x -= x0``; ``y -= y0``).  Random generators are not
compacted (their values come from the RNG stream, not a formula).
"""
from __future__ import annotations

import inspect

import numpy as np
import torch

from . import _lib as L
from . import profiles as P


class GenMask:
    """A compact mask: device table plus its lp mask type code."""

    __slots__ = ("table", "code", "name")

    def __init__(self, table: torch.Tensor, code: int, name: str):
        self.table, self.code, self.name = table, code, name


def _axes(x, y):
    xs = np.asarray(x, dtype=np.float64).reshape(-1)
    ys = np.asarray(y, dtype=np.float64).reshape(-1)
    return xs, ys


def _sep(fx, fy, device, name):
    t = np.concatenate([np.asarray(fx, dtype=np.float64), np.asarray(fy, dtype=np.float64)])
    return GenMask(torch.as_tensor(t.astype(np.float32), device=device), L.LP_MASK_SEP_F32, name)


def round_hole_spans(xs, ys, R, x0=0.0, y0=0.0):
    """(lo, hi) per column of the reference's round_hole mask on the grid
    xs (columns) x ys (rows, ascending): rows lo[j] <= i < hi[j] are inside."""
    thr = 1 / np.exp(0.5)
    xc = xs - x0
    yc = ys - y0
    n_rows = ys.size
    r2 = R ** 2

    def inside(i, j):  # the reference's test (profiles.py:74-81), elementwise
        return np.exp(-(xc[j] ** 2 + yc[i] ** 2) / r2) >= thr

    with np.errstate(invalid="ignore"):
        yw = np.sqrt(np.maximum(r2 / 2 - xc ** 2, 0.0))
    lo0 = np.searchsorted(yc, -yw, side="left")
    hi0 = np.searchsorted(yc, yw, side="right")
    mid = np.full(xs.size, np.searchsorted(yc, 0.0))
    cols = np.arange(xs.size)
    offs = np.arange(-3, 4)
    win = np.concatenate([lo0[:, None] + offs, hi0[:, None] + offs, mid[:, None] + offs], axis=1)
    win = np.clip(win, 0, n_rows - 1)
    ok = inside(win, cols[:, None])
    big = np.where(ok, win, n_rows)
    small = np.where(ok, win, -1)
    lo = big.min(axis=1)
    hi = small.max(axis=1) + 1
    empty = ~ok.any(axis=1)
    lo[empty] = 0
    hi[empty] = 0
    return lo.astype(np.int32), hi.astype(np.int32)


def compact(f_gen, fargs, x, y, device, allow_span: bool = True):
    """GenMask for ``f_gen(x, y, *fargs)`` if f_gen is one of the
    deterministic profile generators, else None.  ``x`` / ``y`` are the
    caller's coordinate arrays (a row and a column, possibly views of one
    array, as Beam2D's X and Y are); gaussian_beam shifts them in place."""
    known = {P.plane_wave, P.gaussian_beam, P.round_hole, P.rectangle_hole, P.square_hole,
             P.square_slits}
    if f_gen not in known or isinstance(x, torch.Tensor) or isinstance(y, torch.Tensor):
        return None
    try:
        ba = inspect.signature(f_gen).bind(x, y, *fargs)
    except TypeError:
        return None
    ba.apply_defaults()
    a = ba.arguments
    if f_gen is P.plane_wave:
        xs, ys = _axes(x, y)
        return _sep(np.ones(xs.size), np.ones(ys.size), device, "plane_wave")
    if f_gen is P.gaussian_beam:
        x -= a["x0"]  # the reference's in-place shift of the caller's grids
        y -= a["y0"]
        xs, ys = _axes(x, y)
        rho2 = a["rho0"] ** 2
        return _sep(a["A0"] * np.exp(-(xs ** 2) / rho2), np.exp(-(ys ** 2) / rho2), device,
                    "gaussian_beam")
    xs, ys = _axes(x, y)
    if f_gen is P.rectangle_hole:
        fx = np.abs(xs - a["x0"]) < (a["dx"] / 2)
        fy = np.abs(ys - a["y0"]) < (a["dy"] / 2)
        return _sep(fx, fy, device, "rectangle_hole")
    if f_gen is P.square_hole:
        d = a["d"]
        return _sep(np.abs(xs - a["x0"]) < (d / 2), np.abs(ys - a["y0"]) < (d / 2), device,
                    "square_hole")
    if f_gen is P.square_slits:
        d, dl = a["d"], a["slits_distance"] / 2
        fx = (np.abs(xs - (a["x0"] - dl)) < (d / 2)) | (np.abs(xs - (a["x0"] + dl)) < (d / 2))
        fy = np.abs(ys - a["y0"]) < (d / 2)
        return _sep(fx, fy, device, "square_slits")
    if f_gen is P.round_hole:
        if not allow_span or np.any(np.diff(ys) <= 0):
            return None
        lo, hi = round_hole_spans(xs, ys, a["R"], a["x0"], a["y0"])
        t = torch.as_tensor(np.concatenate([lo, hi]), device=device)
        return GenMask(t, L.LP_MASK_SPAN_I32, "round_hole")
    return None


def dense(gm: GenMask, n: int) -> torch.Tensor:
    """The N x N float32 mask a GenMask stands for (tests and debugging)."""
    t = gm.table
    if gm.code == L.LP_MASK_SEP_F32:
        return t[n:, None] * t[None, :n]
    rows = torch.arange(n, device=t.device)[:, None]
    return ((rows >= t[None, :n]) & (rows < t[None, n:])).to(torch.float32)
