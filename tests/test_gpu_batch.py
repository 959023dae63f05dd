"""GPU: many beams of uneven sizes in one persistent launch (lp_batch_*).

Each beam of a batch runs lens -> propagate -> iprofile on its own grid; the
result must match the oracle's Beam2D restatement (lens, propagate, |field|^2)
beam by beam, for every grid size the batch accepts, across repeated runs
(the launch resets its own queue) and CUDA-graph replays.  The bounded waits
are exercised with a dependency that nothing satisfies: the run must give up
with a status, not hang, and the next batch must run normally.
"""
import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm, mm, cm = O.um, O.nm, O.mm, O.cm
TOL = 1e-5


@pytest.fixture(scope="module")
def lpb():
    from lightprop2d_gb300 import batch, _lib
    _lib.load()
    return batch


def make_beams(sizes, seed):
    """Seeded per-beam inputs: random-phase round hole, area, wl, z, lens f."""
    rng = np.random.default_rng(seed)
    beams = []
    for i, n in enumerate(sizes):
        area = float(rng.uniform(200 * um, 2 * mm))
        radius = float(rng.uniform(0.05, 0.4)) * area
        wl = float(rng.choice([532 * nm, 632 * nm, 1064 * nm]))
        z = float(rng.uniform(0.5, 20) * cm)
        f = float(rng.uniform(1, 20) * cm) if i % 3 else 0.0
        f0 = O.random_phase_hole(n, area, radius, seed=seed * 1000 + i)
        beams.append(dict(n=n, area=area, wl=wl, z=z, f=f, f0=f0))
    return beams


def oracle_out(b, times=1):
    g = O.grids(b["area"], b["n"], b["wl"])
    x = b["f0"].astype(np.complex128)
    for _ in range(times):
        if b["f"]:
            x, _ = O.lens(x, g["X"], g["Y"], g["k0"], b["f"])
        _, x = O.propagate(O.fft2(x), g["Kz"], b["z"])
    return x


def to_dev(beams):
    fields = [torch.from_numpy(b["f0"].astype(np.complex64)).cuda() for b in beams]
    ips = [torch.empty(b["n"], b["n"], dtype=torch.float32, device="cuda") for b in beams]
    return fields, ips


def make_batch(lpb, beams, fields, ips, **kw):
    return lpb.BeamBatch(fields, [b["area"] for b in beams], [b["wl"] for b in beams],
                         [b["z"] for b in beams], [b["f"] for b in beams], ips, **kw)


def check(beams, fields, ips, times=1):
    torch.cuda.synchronize()
    for b, f, ip in zip(beams, fields, ips):
        ref = oracle_out(b, times)
        got = f.cpu().numpy()
        # each chained application adds its own complex64 rounding
        assert O.rel_l2(got, ref) < TOL * times, (b["n"], O.rel_l2(got, ref))
        if ip is not None:
            ri = O.iprofile(ref)
            e = np.linalg.norm(ip.cpu().numpy() - ri) / np.linalg.norm(ri)
            assert e < 2 * TOL * times, (b["n"], e)


SIZES = [64, 2048, 256, 128, 512, 256, 1024, 64, 4096, 256, 512, 128]


def test_mixed_sizes_parity(lpb):
    beams = make_beams(SIZES, seed=11)
    fields, ips = to_dev(beams)
    bb = make_batch(lpb, beams, fields, ips)
    info = bb.info()
    assert info["items"] > 0 and info["grid"] > 0
    bb.run()
    bb.status()
    check(beams, fields, ips)
    bb.close()


@pytest.mark.parametrize("opts", [dict(tiles_per_item=1, group_points_log2=16),
                                  dict(tiles_per_item=32, group_points_log2=30),
                                  dict(ctas_per_sm=1, tiles_per_item=3)])
def test_options_do_not_change_results(lpb, opts):
    beams = make_beams([512, 128, 1024, 256, 64, 256], seed=12)
    fields, ips = to_dev(beams)
    bb = make_batch(lpb, beams, fields, ips, **opts)
    bb.run()
    bb.status()
    check(beams, fields, ips)


def test_repeated_runs_reset_the_queue(lpb):
    beams = make_beams([256, 1024, 128, 256, 512], seed=13)
    fields, ips = to_dev(beams)
    bb = make_batch(lpb, beams, fields, ips)
    bb.run()
    bb.run()            # second run applies lens + propagate once more
    bb.status()
    check(beams, fields, ips, times=2)


def test_graph_replay(lpb):
    beams = make_beams([512, 256, 2048, 64, 128], seed=14)
    fields, ips = to_dev(beams)
    bb = make_batch(lpb, beams, fields, ips)
    g = bb.capture()    # capture does not execute
    torch.cuda.synchronize()
    for b, f in zip(beams, fields):
        assert np.array_equal(f.cpu().numpy(), b["f0"].astype(np.complex64))
    g.replay()
    bb.status()
    check(beams, fields, ips, times=1)
    g.replay()
    bb.status()
    check(beams, fields, ips, times=2)


def test_without_iprofile_and_flags(lpb):
    beams = make_beams([256, 128], seed=15)
    fields, _ = to_dev(beams)
    bb = lpb.BeamBatch(fields, [b["area"] for b in beams], [b["wl"] for b in beams],
                       [b["z"] for b in beams], [b["f"] for b in beams], None)
    bb.run()
    bb.status()
    check(beams, fields, [None, None])


def test_single_beam_matches_fused_propagate(lpb):
    """A one-beam batch equals the per-size fused kernels (lp_propagate_field)."""
    from lightprop2d_gb300 import backend as B
    b = make_beams([1024], seed=16)[0]
    fields, ips = to_dev([b])
    ref = torch.empty_like(fields[0])
    B.propagate_field(fields[0].clone(), b["area"], b["wl"], b["z"], out=ref, lens_f=b["f"])
    bb = make_batch(lpb, [b], fields, ips)
    bb.run()
    bb.status()
    torch.cuda.synchronize()
    assert O.rel_l2(fields[0].cpu().numpy(), ref.cpu().numpy()) < 2e-6


def test_bounded_wait_gives_up_then_next_batch_runs(lpb):
    from lightprop2d_gb300 import _lib as L
    beams = make_beams([256, 512, 128], seed=17)
    fields, ips = to_dev(beams)
    bad = make_batch(lpb, beams, [f.clone() for f in fields], None,
                     spin_limit=2000, debug_unsatisfiable=True)
    bad.run()
    with pytest.raises(L.BackendError, match="gave up"):
        bad.status()
    # the same plan runs again (its counters were cleared) and gives up again
    bad.run()
    with pytest.raises(L.BackendError):
        bad.status()
    bad.close()
    good = make_batch(lpb, beams, fields, ips)
    good.run()
    good.status()
    check(beams, fields, ips)


def test_invalid_inputs(lpb):
    f = torch.zeros(256, 256, dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError):
        lpb.BeamBatch([], 1.0, 1e-4, 1.0)
    with pytest.raises(ValueError):
        lpb.BeamBatch([torch.zeros(32, 32, dtype=torch.complex64, device="cuda")], 1.0, 1e-4, 1.0)
    with pytest.raises(ValueError):
        lpb.BeamBatch([f], 1.0, 1e-4, [1.0, 2.0])
    with pytest.raises(ValueError):
        lpb.BeamBatch([f], -1.0, 1e-4, 1.0)
    with pytest.raises(ValueError):
        lpb.BeamBatch([f], 1.0, 1e-4, 1.0, flags=0x4)
    with pytest.raises(ValueError):
        lpb.BeamBatch([f.to(torch.complex128)], 1.0, 1e-4, 1.0)


def test_moments_in_last_pass(lpb):
    """Per-beam centroid and D4sigma summed in the batch's last pass match the
    oracle's restatement of Beam2D.centroid / D4sigma on each result, and are
    re-zeroed by every run (graph replays)."""
    beams = make_beams([512, 256, 1024, 128, 2048], seed=21)
    fields, ips = to_dev(beams)
    bb = make_batch(lpb, beams, fields, ips, moments=True)
    g = bb.capture()
    for _ in range(2):
        g.replay()
        bb.status()
        met = bb.metrics()
        for k, (b, f) in enumerate(zip(beams, fields)):
            x = f.cpu().numpy().astype(np.complex128)
            dL = b["area"] / b["n"]
            Xc, Yc, _, _ = O.centroid(x, dL)
            dx, dy = O.d4sigma(x, dL)
            assert abs(met[k, 0] - Xc) < 1e-4 * dL and abs(met[k, 1] - Yc) < 1e-4 * dL, k
            assert np.allclose(met[k, 2:], [dx, dy], rtol=1e-4), (k, met[k], dx, dy)
