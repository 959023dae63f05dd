"""Autotuner: picks launch shapes by timing them on the device.

* ``autotune_propagate(n)`` -- resident CTAs per SM of the row and column pass
  kernels of size n (``lp_tune_ctas_per_sm``), measured on the fused
  field -> field propagate; the best pair stays in effect for the process.
* ``autotune_batch(...)`` -- for a batch of uneven beams: CTAs per SM, tiles
  per queue item and scheduling-group size of the persistent batch launch.
  Results are cached per batch signature (histogram of grid sizes).

Timings are CUDA events on the launching stream, median of ``reps`` runs
after a warm-up.  The radix schedule per size is fixed (16 x 16 x R); the
tuner chooses how the work is laid onto the GB300's SMs.
"""
from __future__ import annotations

import itertools
import statistics
from collections import Counter

import torch

from . import _lib as L
from . import backend as B
from .batch import BeamBatch

_batch_cache: dict = {}


def _time(fn, reps, stream):
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        out.append((a, b))
    torch.cuda.synchronize()
    return statistics.median(a.elapsed_time(b) for a, b in out)


def autotune_propagate(n: int, area_size: float = 0.2, wl: float = 632e-7, z: float = 1.0,
                       reps: int = 30, max_ctas: int = 8, apply: bool = True):
    """Time the fused propagate of size n for every (row, column) CTAs-per-SM
    setting; returns (best (row, col), {setting: ms}) and keeps the best in
    effect when ``apply``."""
    lib = L.load()
    B.init()
    st = torch.cuda.current_stream()
    x = torch.randn(n, n, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    res = {}
    for r, c in itertools.product(range(1, max_ctas + 1), range(1, max_ctas + 1)):
        er = lib.lp_tune_ctas_per_sm(n, 0, r)
        ec = lib.lp_tune_ctas_per_sm(n, 1, c)
        if (er, ec) in res:
            continue
        res[(er, ec)] = _time(lambda: B.propagate_field(x, area_size, wl, z, out=y), reps, st)
    best = min(res, key=res.get)
    lib.lp_tune_ctas_per_sm(n, 0, best[0] if apply else 0)
    lib.lp_tune_ctas_per_sm(n, 1, best[1] if apply else 0)
    return best, res


def batch_signature(fields) -> tuple:
    return tuple(sorted(Counter(int(f.shape[0]) for f in fields).items()))


def autotune_batch(fields, area_size, wl, z, lens_f=0.0, iprofiles=None, reps: int = 3,
                   ctas=(1, 2), tiles_per_item=(4, 8, 16), group_points_log2=(21, 22, 23, 24)):
    """Time the batch for every candidate option set and return
    (best options dict, {options tuple: ms}).  The fields are transformed in
    place by every timed run: pass scratch copies.  Cached per signature."""
    sig = batch_signature(fields)
    if sig in _batch_cache:
        return _batch_cache[sig]
    st = torch.cuda.current_stream()
    res = {}
    for c, t, g in itertools.product(ctas, tiles_per_item, group_points_log2):
        b = BeamBatch(fields, area_size, wl, z, lens_f, iprofiles, ctas_per_sm=c,
                      tiles_per_item=t, group_points_log2=g)
        res[(c, t, g)] = _time(b.run, reps, st)
        b.status()
        b.close()
    best = min(res, key=res.get)
    out = ({"ctas_per_sm": best[0], "tiles_per_item": best[1], "group_points_log2": best[2]},
           res)
    _batch_cache[sig] = out
    return out
