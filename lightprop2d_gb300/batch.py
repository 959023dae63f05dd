"""Many beams of uneven sizes in one persistent launch (lp_batch_* C ABI).

Each beam runs ``lens(lens_f) -> propagate(z) -> iprofile`` in place on its
own grid -- the reference's ``Beam2D.lens`` + ``Beam2D.propagate`` +
``Beam2D.iprofile`` (lightprop2d/beam2d.py:492-511, :462-490, :706-721) --
and the whole batch is one kernel launch, optionally captured in a CUDA graph.

``partition_beams`` splits a batch across ranks (one GPU each) by points with
no collective: beams are independent, so multi-GPU is replicas of this launch
over disjoint shards.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from . import _lib as L


class BeamBatch:
    """A planned batch.  ``fields`` are complex64 CUDA (n, n) tensors that are
    transformed in place; ``iprofiles`` (optional) float32 (n, n) outputs.

    Scalars may be given per beam (sequences) or once for all beams.
    """

    def __init__(self, fields: Sequence[torch.Tensor], area_size, wl, z, lens_f=0.0,
                 iprofiles: Sequence[torch.Tensor] | None = None, flags: int = 0,
                 ctas_per_sm: int = 0, tiles_per_item: int = 0, group_points_log2: int = 0,
                 spin_limit: int = 0, debug_unsatisfiable: bool = False,
                 moments: bool = False):
        nb = len(fields)
        if nb == 0:
            raise ValueError("empty batch")

        def per(v, name):
            if isinstance(v, (list, tuple)):
                if len(v) != nb:
                    raise ValueError(f"{name}: expected {nb} values")
                return [float(x) for x in v]
            return [float(v)] * nb

        areas, wls, zs, fs = per(area_size, "area_size"), per(wl, "wl"), per(z, "z"), \
            per(lens_f, "lens_f")
        descs = (L.BeamDesc * nb)()
        self.fields = list(fields)
        self.areas = areas
        # per-beam intensity moments summed in the last pass (see metrics())
        self.moments = (torch.zeros((nb, 5), dtype=torch.float64, device=self.fields[0].device)
                        if moments else None)
        self.iprofiles = list(iprofiles) if iprofiles is not None else [None] * nb
        dev = self.fields[0].device
        for i, f in enumerate(self.fields):
            if not (f.is_cuda and f.dtype == torch.complex64 and f.dim() == 2
                    and f.shape[0] == f.shape[1] and f.is_contiguous() and f.device == dev):
                raise ValueError(f"field {i}: complex64 contiguous square CUDA tensor on {dev}")
            ip = self.iprofiles[i]
            if ip is not None and not (ip.is_cuda and ip.dtype == torch.float32
                                       and tuple(ip.shape) == tuple(f.shape)):
                raise ValueError(f"iprofile {i}: float32 CUDA tensor of the field's shape")
            mp = self.moments[i].data_ptr() if self.moments is not None else 0
            descs[i] = L.BeamDesc(f.data_ptr(), ip.data_ptr() if ip is not None else 0,
                                  f.shape[0], areas[i], wls[i], zs[i], fs[i], int(flags), mp)
        opts = L.BatchOptions(int(ctas_per_sm), int(tiles_per_item), int(group_points_log2),
                              int(spin_limit), int(bool(debug_unsatisfiable)))
        self.device = dev
        self._lib = L.load()
        handle = ctypes.c_void_p()
        with torch.cuda.device(dev):
            L.check(self._lib.lp_batch_create(descs, nb, ctypes.byref(opts), ctypes.byref(handle)),
                    "lp_batch_create")
        self._h = handle
        self.n_points = sum(f.shape[0] * f.shape[1] for f in self.fields)

    def _stream(self, stream):
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        return ctypes.c_void_p(s.cuda_stream)

    def run(self, stream=None) -> None:
        """One persistent launch over the whole batch (asynchronous)."""
        with torch.cuda.device(self.device):
            L.check(self._lib.lp_batch_run(self._h, self._stream(stream)), "lp_batch_run")

    def status(self, stream=None) -> None:
        """Synchronise and raise if a bounded device-side wait gave up."""
        with torch.cuda.device(self.device):
            L.check(self._lib.lp_batch_status(self._h, self._stream(stream)), "lp_batch_status")

    def info(self) -> dict:
        n, g, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.check(self._lib.lp_batch_info(self._h, ctypes.byref(n), ctypes.byref(g),
                                        ctypes.byref(c)), "lp_batch_info")
        return {"items": n.value, "grid": g.value, "ctas_per_sm": c.value}

    def metrics(self):
        """Per-beam (Xc, Yc, D4sigma_x, D4sigma_y) in cm after a run, from the
        moments summed in the last pass (Beam2D.centroid / D4sigma,
        beam2d.py:669-704).  The widths use raw moments about the grid
        centre: the relative error grows like (offset / width)^2 * 1e-7, so
        beams far off centre relative to their width should use
        Beam2D.D4sigma (second moments about the centroid)."""
        if self.moments is None:
            raise ValueError("BeamBatch(..., moments=True) is needed for metrics()")
        m = self.moments.cpu().numpy()
        n = np.array([f.shape[0] for f in self.fields], dtype=np.float64)
        dL = np.asarray(self.areas, dtype=np.float64) / n
        with np.errstate(invalid="ignore", divide="ignore"):
            xc, yc = m[:, 1] / m[:, 0], m[:, 2] / m[:, 0]
            vx = np.maximum(m[:, 3] / m[:, 0] - xc ** 2, 0.0)
            vy = np.maximum(m[:, 4] / m[:, 0] - yc ** 2, 0.0)
        return np.stack([dL * xc, dL * yc, 4 * dL * np.sqrt(vx), 4 * dL * np.sqrt(vy)], axis=1)

    def capture(self) -> torch.cuda.CUDAGraph:
        """Capture one run into a CUDA graph (replay with graph.replay())."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.run(stream=s)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_info(sizes: Sequence[int], area_size, wl, z, lens_f=0.0, flags: int = 0,
              tiles_per_item: int = 0, group_points_log2: int = 0) -> dict:
    """The work queue lp_batch_create would build for beams of these grid
    sizes (host only, no CUDA call: lp_batch_plan).  Field pointers are
    placeholders; only the plan is computed.  Returns items, tiles, points."""
    nb = len(sizes)
    if nb == 0:
        raise ValueError("empty batch")

    def per(v):
        return [float(x) for x in v] if isinstance(v, (list, tuple)) else [float(v)] * nb
    areas, wls, zs, fs = per(area_size), per(wl), per(z), per(lens_f)
    descs = (L.BeamDesc * nb)()
    for i, n in enumerate(sizes):
        # placeholder addresses: aligned, never dereferenced by the planner
        descs[i] = L.BeamDesc(4096 * (i + 1), 0, int(n), areas[i], wls[i], zs[i], fs[i],
                              int(flags), 0)
    opts = L.BatchOptions(0, int(tiles_per_item), int(group_points_log2), 0, 0)
    items, tiles, points = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
    L.check(L.load().lp_batch_plan(descs, nb, ctypes.byref(opts), ctypes.byref(items),
                                   ctypes.byref(tiles), ctypes.byref(points)), "lp_batch_plan")
    return {"items": items.value, "tiles": tiles.value, "points": points.value}


def shard(sizes: Sequence[int], world: int, rank: int) -> list[int]:
    """The beam indices rank `rank` of `world` propagates (partition_beams)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return partition_beams(sizes, world)[rank]


def partition_beams(sizes: Sequence[int], world: int) -> list[list[int]]:
    """Split beams (grid sizes n) over `world` ranks, balancing points:
    longest-processing-time greedy (largest beam to the lightest rank).
    Deterministic; every beam lands on exactly one rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]) ** 2, i))
    loads = [0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += int(sizes[i]) ** 2
    for p in parts:
        p.sort()
    return parts
