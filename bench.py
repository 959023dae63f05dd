"""Benchmark: 2048^2 complex64 angular-spectrum propagates/s on one GB300.

Workload (``config.workload``): Gaussian beam, npoints=2048, area 2 mm,
wl 632 nm, waist 100 um, complex64, propagated by z = 1 cm per step.  A step
is one fused field -> field propagate (fft2 -> H(z) in registers -> ifft2,
read field / write field) with the field resident in HBM.  L2 hygiene: the
timed steps rotate over in/out grid pairs totalling > 2.5x the L2, so no step
finds its input in L2 (a 320 MiB-flush variant is reported beside it).

Also reported: the per-pass breakdown, the Beam2D.propagate steady state
(stored spectrum -> field), the plain unfused form (fft2, H grid in HBM,
multiply, ifft2) with the float-float H and with the reference-literal FP64
H, the plain-FP32-phase variant's error by z, an N sweep (512..4096), the
phase-mask inverse design and split-step chain workloads, the 4096-beam
uneven batch (one persistent launch in a CUDA graph, autotuned, against
per-beam calls) and ``e2e``: the same step through the C ABI with host
buffers (pinned H2D copy, propagate, D2H copy timed).

``--impl reference`` times the reference algorithm (the numpy oracle port of
beam2d.py:481-490 with the fft2 of the field first) on the host cores, one
process per core, on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_HEAD, AREA, WL, WAIST, Z = 2048, 0.2, 632e-7, 100e-4, 1.0
# DRAM bytes per launch of the 2048^2 pass kernels, measured with ncu on this
# workload with caches kept warm between launches (a live step's L2 state):
# the column pass reads its input from L2 and only writes back evictions.
NCU_DRAM_BYTES_2048 = {"row_fwd": 59.22e6, "col_fwd_H_inv": 16.91e6, "row_inv": 0.69e6}
# The same kernels' FP32 (FMA) pipe and issue activity from an ncu --set full
# capture of this workload: the FFT passes are bound on-chip, not by DRAM.
NCU_PIPES_2048 = {"col_fwd_H_inv": {"fma_pipe_active_pct": 33.1, "issue_active_pct": 48.4},
                  "row_fwd": {"fma_pipe_active_pct": 21.5, "issue_active_pct": 30.2},
                  "row_inv": {"fma_pipe_active_pct": 21.6, "issue_active_pct": 30.3}}
METRIC = "2048^2 complex64 fused field->field propagates/s"
UNIT = "propagates/s"
WORKLOAD = "gaussian beam 2048^2, area 2 mm, wl 632 nm, waist 100 um, complex64, z=1 cm/step"
L2_NOTE = "inputs larger than L2: timed steps rotate over in/out grid pairs totalling > 2.5x the 126 MB L2"


def bench_config():
    """The `config` both arms print (identical, so the runs compare)."""
    return {"workload": WORKLOAD, "l2": L2_NOTE}


# ----------------------------------------------------------------- CPU side --
def _cpu_worker_init(n, area, wl):
    global _W
    import numpy as _np
    from oracle import lp_oracle as O
    g = O.grids(area, n, wl)
    f = O.gaussian(n, area, 1.0, WAIST).astype(_np.complex64)
    _W = (g["Kz"], f)


def _cpu_worker_step(z):
    """One field -> field propagate exactly as the reference computes it:
    spectrum = fft2(field) (beam2d.py:217), spectrum *= H (:485-489),
    field = ifft2(spectrum) (:490), complex64 arrays, FP64 phase."""
    import numpy as _np
    from oracle import lp_oracle as O
    Kz, f = _W
    t0 = time.perf_counter()
    s = _np.fft.fft2(f)
    s, out = O.propagate(s, Kz, z)
    dt = time.perf_counter() - t0
    return dt, float(_np.abs(out[0, 0]))


def cpu_baseline(steps: int, n=N_HEAD, procs=None, warmup=3):
    """Run `warmup` untimed then `steps` timed rounds; each round every
    process propagates one beam."""
    # LP_BENCH_CPU_PROCS caps the processes (default: one per host core)
    procs = procs or int(os.environ.get("LP_BENCH_CPU_PROCS", "0")) or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=_cpu_worker_init, initargs=(n, AREA, WL)) as pool:
        for _ in range(max(1, warmup)):
            pool.map(_cpu_worker_step, [Z] * procs)
        walls = []
        for _ in range(steps):
            t0 = time.perf_counter()
            pool.map(_cpu_worker_step, [Z] * procs)
            walls.append(time.perf_counter() - t0)
    total = procs * steps
    return dict(value=total / sum(walls), unit=UNIT, cores=procs, kind="port",
                sample=f"{total} field->field propagates at {n}^2 complex64 "
                       f"({procs} processes x {steps} rounds, numpy pocketfft)")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    # a step is one round: every host core propagates one 2048^2 beam
    # (~0.2-0.9 s); the requested steps are run (capped at 200 rounds)
    steps = max(1, min(args.steps, 200))
    warmup = max(3, min(args.warmup, 20))
    cb = cpu_baseline(steps, warmup=warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
        "ms_per_step": 1000.0 / cb["value"] * cb["cores"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": bench_config(), "parallelism": "host processes (one per core)",
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------ batch workload --
# 4096 beams: 64% 256^2, 25% 512^2, 9% 1024^2, 2% 2048^2 (1,171,062,784 points).
BATCH_MIX = ((256, 2621), (512, 1024), (1024, 369), (2048, 82))
BATCH_WL = 632e-7


def batch_workload(dev, seed=3, mix=BATCH_MIX, scale=1.0):
    """Seeded uneven-size batch, generated on the device: per beam a round
    hole of radius U[0.05, 0.40]*A (amplitude U[0,1), phase U[0,2pi)), area
    A = U[200 um, 2 mm], lens f = U[1, 20] cm, z = U[0.5, 20] cm, wl 632 nm.
    Beams of one size are slices of one (count, n, n) tensor.  Returns a dict
    of per-beam lists (fields, iprofiles, area, z, f, n)."""
    import torch
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    out = {k: [] for k in ("fields", "iprofiles", "area", "z", "f", "n")}
    out["stacks"] = []
    for n, cnt in mix:
        cnt = max(1, int(round(cnt * scale)))
        frac = rng.uniform(0.05, 0.40, cnt)
        out["area"] += list(rng.uniform(200e-4, 0.2, cnt))
        out["f"] += list(rng.uniform(1.0, 20.0, cnt))
        out["z"] += list(rng.uniform(0.5, 20.0, cnt))
        st = torch.empty(cnt, n, n, dtype=torch.complex64, device=dev)
        ip = torch.empty(cnt, n, n, dtype=torch.float32, device=dev)
        j = torch.arange(-n // 2, n // 2, device=dev, dtype=torch.float64)
        r2 = j[None, :] ** 2 + j[:, None] ** 2          # (x^2 + y^2) / dL^2
        chunk = max(1, (1 << 25) // (n * n))
        for c0 in range(0, cnt, chunk):
            c1 = min(cnt, c0 + chunk)
            amp = torch.rand(c1 - c0, n, n, generator=gen, device=dev)
            ph = torch.rand(c1 - c0, n, n, generator=gen, device=dev) * (2 * np.pi)
            thr = torch.as_tensor((frac[c0:c1] * n) ** 2, device=dev)  # (radius/dL)^2
            amp = amp * (r2[None] <= thr[:, None, None])
            st[c0:c1] = torch.polar(amp, ph)
        out["stacks"].append((st, ip))
        out["fields"] += [st[i] for i in range(cnt)]
        out["iprofiles"] += [ip[i] for i in range(cnt)]
        out["n"] += [n] * cnt
    return out


def batch_section(dev, stream, clocks, reps, check_oracle=True, scale=1.0, compare=True,
                  shard_of=None):
    """Config: the uneven batch as one persistent launch in a CUDA graph
    (autotuned options), against the same beams as per-beam fused calls.
    Parity: sampled beams against the oracle, and for every beam energy
    conservation (the lens and H are unimodular: sum |u|^2 before equals
    sum of the iprofile after, to FFT round-off).  shard_of = (world, rank):
    only this rank's share of the beams (batch.shard: points balanced, no
    collective), as a multi-GPU run splits the batch."""
    import torch
    from lightprop2d_gb300 import _lib as L
    from lightprop2d_gb300 import backend as B
    from lightprop2d_gb300 import tune
    from lightprop2d_gb300.batch import BeamBatch
    from oracle import lp_oracle as O

    W = batch_workload(dev, scale=scale)
    e_in = torch.cat([(st.real ** 2 + st.imag ** 2).sum((1, 2), dtype=torch.float64)
                      for st, _ in W["stacks"]])
    own = None
    if shard_of is not None:
        from lightprop2d_gb300.batch import shard
        own = shard(W["n"], *shard_of)
        for k in ("fields", "iprofiles", "area", "z", "f", "n"):
            W[k] = [W[k][i] for i in own]
        e_in = e_in[torch.as_tensor(own, device=e_in.device)]
    nb, pts = len(W["fields"]), sum(n * n for n in W["n"])
    # parity sample: first beam of every size, kept on the host before any run
    pick = [W["n"].index(n) for n, _ in BATCH_MIX if n in W["n"]]
    keep = {i: W["fields"][i].cpu().numpy() for i in pick}
    args = (W["area"], BATCH_WL, W["z"], W["f"], W["iprofiles"])
    bb = BeamBatch(W["fields"], *args)
    bb.run()
    bb.status()
    torch.cuda.synchronize()
    errs = {}
    if check_oracle:
        for i in pick:
            n = W["n"][i]
            g = O.grids(W["area"][i], n, BATCH_WL)
            x, _ = O.lens(keep[i].astype(np.complex128), g["X"], g["Y"], g["k0"], W["f"][i])
            _, x = O.propagate(O.fft2(x), g["Kz"], W["z"][i])
            errs[str(n)] = O.rel_l2(W["fields"][i].cpu().numpy(), x)
    e_out = torch.cat([ip.sum((1, 2), dtype=torch.float64) for _, ip in W["stacks"]])
    if own is not None:
        e_out = e_out[torch.as_tensor(own, device=e_out.device)]
    energy_err = float(((e_out - e_in).abs() / e_in).max())
    bb.close()
    del keep

    if compare:
        with clocks.window():
            best, table = tune.autotune_batch(W["fields"], *args, reps=3)
    else:
        best, table = {}, {}
    bb = BeamBatch(W["fields"], *args, **best)
    info = bb.info()
    graph = bb.capture()

    def ev_time(fn, k):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(k):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k

    with clocks.window():
        t_graph = ev_time(graph.replay, reps)
    bb.status()
    # the same batch with per-beam intensity moments summed in the last pass
    bm = BeamBatch(W["fields"], *args, **best, moments=True)
    gm = bm.capture()
    with clocks.window():
        t_moments = ev_time(gm.replay, max(3, reps // 2))
    bm.status()
    bm.close()
    del gm

    if not compare:
        bb.close()
        del graph
        return {"beams": nb, "points": pts, "ms_per_batch": round(t_graph, 4),
                "ms_per_batch_with_moments": round(t_moments, 4), "plan": info,
                "energy_rel_err_max_all_beams": energy_err, "rel_l2_vs_fp64_oracle": errs}

    # the same beams as one fused field->field call each (3 launches per beam)
    fl, ipl = W["fields"], W["iprofiles"]

    def per_beam():
        for i in range(nb):
            B.propagate_field(fl[i], W["area"][i], BATCH_WL, W["z"][i], out=fl[i],
                              iprofile_out=ipl[i], lens_f=W["f"][i])

    with clocks.window():
        t_calls = ev_time(per_beam, max(2, reps // 4))
        g2 = torch.cuda.CUDAGraph()
        s2 = torch.cuda.Stream(device=dev)
        s2.wait_stream(stream)
        with torch.cuda.stream(s2):
            with torch.cuda.graph(g2, stream=s2):
                per_beam()
        stream.wait_stream(s2)
        t_calls_graph = ev_time(g2.replay, max(2, reps // 2))
    bb.close()
    del graph, g2
    alg = 20 * pts  # field read + write, iprofile write
    return {
        "workload": "4096 beams: " + ", ".join(f"{c} x {n}^2" for n, c in BATCH_MIX)
                    + f" ({pts} points), hole+lens+propagate+iprofile, wl 632 nm",
        "beams_per_s": round(nb / (t_graph * 1e-3), 1),
        "points_per_s": round(pts / (t_graph * 1e-3), 1),
        "ms_per_batch": round(t_graph, 4),
        "effective_gbs": round(alg / (t_graph * 1e-3) / 1e9, 1),
        "alg_bytes_per_batch": alg,
        "launches_per_batch": 1,
        "ms_per_batch_with_moments": round(t_moments, 4),
        "plan": {**best, **info},
        "autotune_ms": {str(k): round(v, 4) for k, v in table.items()},
        "per_beam_calls_ms": round(t_calls, 4),
        "per_beam_calls_graph_ms": round(t_calls_graph, 4),
        "speedup_vs_per_beam_graph": round(t_calls_graph / t_graph, 3),
        "rel_l2_vs_fp64_oracle": errs,
        "energy_rel_err_max_all_beams": energy_err,
        "l2": f"{pts * 8 / 2**30:.1f} GiB of fields per batch (> L2)",
    }


def next_rows_section(dev, stream, hbm):
    """Per-op device time and effective HBM bandwidth (bytes each op must move
    / time, against the measured copy peak) at 2048^2 unless stated."""
    import torch
    from lightprop2d_gb300 import backend as B
    from lightprop2d_gb300 import generators as G
    from lightprop2d_gb300 import modes as MD
    from lightprop2d_gb300 import profiles as P

    def t_us(fn, k=50):
        """Device time per call: k calls captured in a CUDA graph and replayed,
        so host-side call overhead is not timed."""
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(device=dev)
        s.wait_stream(stream)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(k):
                    fn()
        stream.wait_stream(s)
        g.replay()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        g.replay()
        b.record(stream)
        torch.cuda.synchronize()
        del g
        return a.elapsed_time(b) / k * 1e3

    def row(us, nbytes, note):
        return {"us": round(us, 2), "bytes": int(nbytes),
                "effective_gbs": round(nbytes / (us * 1e-6) / 1e9, 1),
                "hbm_frac": round(nbytes / (us * 1e-6) / 1e9 / hbm, 3), "note": note}

    n = 2048
    f = torch.randn(n, n, dtype=torch.complex64, device=dev)
    out = {}
    mom = torch.empty(5, dtype=torch.float64, device=dev)
    out["beam_moments"] = row(t_us(lambda: B.beam_moments(f, mom)), 8 * n * n,
                              "one read pass + finish (moments about the centroid)")
    # coordinate_filter(f_gen=round_hole) folded into a propagate, vs a dense mask
    X = np.arange(-n // 2, n // 2) * (0.2 / n)
    gm = G.compact(P.round_hole, (0.05,), X.copy(), X.copy().reshape((-1, 1)), dev)
    dense = torch.as_tensor(P.round_hole(X.copy(), X.copy().reshape((-1, 1)), 0.05), device=dev)
    dense = dense.to(torch.uint8)
    o = torch.empty_like(f)
    tg = t_us(lambda: B.propagate_field(f, 0.2, WL, 1.0, out=o, xmask=gm))
    td = t_us(lambda: B.propagate_field(f, 0.2, WL, 1.0, out=o, xmask=dense))
    t0 = t_us(lambda: B.propagate_field(f, 0.2, WL, 1.0, out=o))
    ph = torch.rand(n, n, device=dev) * 6.283
    tl = t_us(lambda: B.propagate_field(f, 0.2, WL, 1.0, out=o, lens_f=5.0))
    tp = t_us(lambda: B.propagate_field(f, 0.2, WL, 1.0, out=o, xmask=ph, xmask_phase=True))
    out["generator_in_pass"] = {"round_hole_table_us": round(tg, 2),
                                "dense_u8_mask_us": round(td, 2), "lens_us": round(tl, 2),
                                "phase_mask_us": round(tp, 2), "no_mask_us": round(t0, 2),
                                "note": "fused propagate with the multiplier in the first pass"}
    del ph
    out["expand"] = row(t_us(lambda: B.expand(f, 2 * n), 20), 8 * n * n + 8 * 4 * n * n,
                        "2048^2 -> 4096^2")
    out["coarse"] = row(t_us(lambda: B.coarse(f, 2)), 8 * n * n + 8 * n * n // 4,
                        "2048^2 -> 1024^2 block mean")
    out["crop"] = row(t_us(lambda: B.crop(f, n // 4, n // 2, -0.05, 0.2 / n, n, 0.1 / n)),
                      8 * n * n // 4 + 8 * n * n, "window 1024^2 resampled to 2048^2")
    M, nb = 256, 1024
    basis = MD.ModeBasis(torch.randn(M, nb * nb, dtype=torch.complex64, device=dev))
    coef = torch.randn(M, dtype=torch.complex128, device=dev)
    out["modes_project"] = row(t_us(lambda: MD.project(basis, f), 10), 8 * M * nb * nb,
                               f"{M} modes x {nb}^2 window of a 2048^2 field")
    out["modes_combine"] = row(t_us(lambda: MD.combine(basis, coef, n, f.device), 10),
                               8 * M * nb * nb + 8 * n * n, f"{M} modes into a 2048^2 field")
    del basis, f, o
    return out


# ----------------------------------------------------------------- GPU side --
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
         "utilization.gpu")

    def __init__(self, index):
        self.index, self.samples, self.windows = index, [], []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [s.strip() for s in line.split(",")]))

    def window(self):
        return _Window(self)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        inside = [s for t, s in self.samples
                  if any(a - 0.15 <= t <= b + 0.15 for a, b in self.windows)]
        use = inside or [s for _, s in self.samples]
        if not use:
            return None
        mhz = [float(s[1]) for s in use if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in use if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in use for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(mhz) if mhz else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(use), "in_timed_region": bool(inside)}


class _Window:
    def __init__(self, cs):
        self.cs = cs

    def __enter__(self):
        self.t0 = time.time()

    def __exit__(self, *a):
        self.cs.windows.append((self.t0, time.time()))


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--quick", action="store_true", help="skip the sweep")
    ap.add_argument("--only", choices=["batch", "next_rows", "propagate", "c128"],
                    help="run one section once and print its JSON (profiling cases)")
    ap.add_argument("--n", type=int, default=2048,
                    help="grid size of --only propagate (fused propagates back to back)")
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="beam counts of the uneven batch times this factor (--only batch)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # --gpus N without a launcher: start N ranks (one per GPU) on this node
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
               f"--nproc-per-node={args.gpus}", "--master-addr=127.0.0.1",
               f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
        return subprocess.call(cmd)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    # CPU baseline first (spawned pool, before any CUDA work in this process).
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu and not args.only:
        cb = cpu_baseline(steps=3)
        one = cpu_baseline(steps=2, procs=1)
        cb["one_process"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from lightprop2d_gb300 import _lib as L
    from lightprop2d_gb300 import backend as B
    from oracle import lp_oracle as O
    lib = L.load()
    B.init(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(320 * 2 ** 20 // 4, dtype=torch.float32, device=dev)

    def vp(t):
        return ctypes.c_void_p(t.data_ptr())

    nul = ctypes.c_void_p(0)

    def fused(n, fin, fout, z=Z, flags=0):
        return lib.lp_propagate_field(vp(fin), vp(fout), nul, nul, n, AREA, WL, z, 0.0,
                                      nul, 0, nul, 0, flags, sp)

    def spec_state(n, s, fout, z=Z):
        return lib.lp_propagate(vp(s), vp(fout), n, AREA, WL, z, nul, 0,
                                L.LP_FLAG_SPECTRUM_READONLY, sp)

    def plain(n, fin, fout, fp64=False):
        return lib.lp_plain_propagate_field(vp(fin), vp(fout), n, AREA, WL, Z,
                                            L.LP_FLAG_PLAIN_FP64_H if fp64 else 0, sp)

    L2_BYTES = 126 * 2 ** 20

    def nslots(n):
        """In/out grid pairs to rotate through: their total is > 2.5x the L2,
        so a step never finds its input (or its output lines) in L2."""
        return int(min(128, max(3, -(-int(2.5 * L2_BYTES) // (16 * n * n)))))

    def make(n, slots=1):
        f = torch.as_tensor(O.gaussian(n, AREA, 1.0, WAIST).astype(np.complex64), device=dev)
        return [(f.clone(), torch.empty_like(f)) for _ in range(slots)]

    ranks_in_step = {"on": True}  # False inside rank-0-only sections (no barriers)

    def timed(fn, steps, warmup, npass=0, flush_l2=False):
        """CUDA-event timing on the launching stream.  fn(i) runs step i.

        L2 hygiene: by default fn rotates over nslots() in/out pairs (inputs
        larger than L2 in total); flush_l2=True instead writes a 320 MiB buffer
        before every step (outside per-step events).  Default (the timing of
        record): one event pair brackets all `steps` back-to-back steps, so
        consecutive launches overlap as they do in use.  flush_l2: two events
        per step.  npass > 0: the library records events at its pass
        boundaries (lp_profile_events), which keeps consecutive passes from
        overlapping their launches -- used only for the per-pass breakdown.
        Returns (per-step ms list, per-pass ms lists)."""
        for i in range(warmup):
            L.check(fn(i), "warm-up")
        torch.cuda.synchronize()
        if not npass and not flush_l2:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if dist and ranks_in_step["on"]:
                dist.barrier()
            torch.cuda.synchronize()
            a.record(stream)
            for i in range(steps):
                L.check(fn(i), "timed step")
            b.record(stream)
            torch.cuda.synchronize()
            if dist and ranks_in_step["on"]:
                dist.barrier()
            tot = a.elapsed_time(b)
            return [tot / steps] * steps, []
        ne = npass + 1 if npass else 2
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(ne)] for _ in range(steps)]
        for row in evs:
            for e in row:
                e.record(stream)
        torch.cuda.synchronize()
        if dist and ranks_in_step["on"]:
            dist.barrier()
        torch.cuda.synchronize()
        for i in range(steps):
            if flush_l2:
                flush.fill_(float(i))
            if npass:
                arr = (ctypes.c_void_p * ne)(*[e.cuda_event for e in evs[i]])
                lib.lp_profile_events(arr, ne)
                L.check(fn(i), "timed step")
            else:
                evs[i][0].record(stream)
                L.check(fn(i), "timed step")
                evs[i][1].record(stream)
        lib.lp_profile_events(None, 0)
        torch.cuda.synchronize()
        if dist and ranks_in_step["on"]:
            dist.barrier()
        step = [row[0].elapsed_time(row[-1]) for row in evs]
        passes = [[row[p].elapsed_time(row[p + 1]) for row in evs] for p in range(npass)]
        return step, passes

    clocks = ClockSampler(local)
    if args.only:
        # one section, once (the cases the committed ncu summaries profile)
        if args.only == "batch":
            res = batch_section(dev, stream, clocks, reps=2, check_oracle=False,
                                scale=args.batch_scale, compare=False)
        elif args.only == "propagate":
            nn = args.n
            rr = nslots(nn)
            sl = make(nn, rr)
            sm, _ = timed(lambda i: fused(nn, *sl[i % rr]), args.steps, args.warmup)
            _, pm = timed(lambda i: fused(nn, *sl[i % rr]), args.steps, 3, 3)
            ms = statistics.fmean(sm)
            res = {"n": nn, "ms": round(ms, 5), "propagates_per_s": round(1e3 / ms, 1),
                   "effective_gbs": round(16 * nn * nn / (ms * 1e-3) / 1e9, 1),
                   "passes_ms": [round(statistics.fmean(p), 5) for p in pm],
                   "slots": rr}
        elif args.only == "c128":
            # complex128 fused propagates back to back (--n grid), and the
            # spectrum-state propagate of Beam2D
            nn = args.n
            zi = torch.as_tensor(O.gaussian(nn, AREA, 1.0, WAIST).astype(np.complex128),
                                 device=dev)
            zo = torch.empty_like(zi)
            zs = torch.fft.fft2(zi)
            zf = torch.empty_like(zi)
            def fused128(i):
                B.propagate_field(zi, AREA, WL, Z, out=zo)
                return 0

            def state128(i):
                B.propagate(zs, AREA, WL, Z, field_out=zf, write_spectrum=False)
                return 0
            fm, _ = timed(fused128, args.steps, args.warmup)
            sm, _ = timed(state128, args.steps, args.warmup)
            res = {"n": nn, "fused_ms": round(statistics.fmean(fm), 5),
                   "spectrum_state_ms": round(statistics.fmean(sm), 5)}
        else:
            res = next_rows_section(dev, stream, peaks()[0])
        print(json.dumps({"section": args.only, **res}))
        return 0
    clocks.start()
    time.sleep(0.3)

    # ---------------------------------------------------------- headline --
    n = N_HEAD
    R = nslots(n)
    slots = make(n, R)
    head = lambda i: fused(n, *slots[i % R])
    with clocks.window():
        step_ms, _ = timed(head, args.steps, args.warmup)
        flush_ms, _ = timed(lambda i: fused(n, *slots[0]), max(10, min(args.steps, 500)), 3,
                            flush_l2=True)
        # per-pass breakdown (events at the pass boundaries), a separate loop
        _, pass_ms = timed(head, max(10, min(args.steps, 500)), 3, 3)
    tot_ms = sum(step_ms)
    if dist:
        t = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t)
    ms_step = tot_ms / args.steps
    value = world * args.steps / (tot_ms / 1e3)

    # parity of a timed result vs the oracle (same step, complex128)
    g = O.grids(AREA, n, WL)
    _, f_ref = O.propagate(np.fft.fft2(O.gaussian(n, AREA, 1.0, WAIST)), g["Kz"], Z)
    torch.cuda.synchronize()
    fout = slots[(args.steps - 1) % R][1]
    err = O.rel_l2(fout.cpu().numpy(), f_ref)
    eerr = O.energy_err(fout.cpu().numpy(), f_ref)

    hbm, peak_kind = peaks()
    pass_avg = [statistics.fmean(p) for p in pass_ms]
    names = ["row_fwd", "col_fwd_H_inv", "row_inv"]
    dom = int(np.argmax(pass_avg))
    alg_bytes = 16 * n * n  # each pass reads and writes one complex64 grid
    achieved = alg_bytes / (pass_avg[dom] * 1e-3) / 1e9
    step_gbs = alg_bytes / (ms_step * 1e-3) / 1e9

    extra = {"passes_ms": dict(zip(names, [round(x, 5) for x in pass_avg])),
             "step_effective_gbs": round(step_gbs, 1),
             "step_roofline_frac": round(step_gbs / hbm, 4),
             "flush_l2_mode": {"ms": round(statistics.fmean(flush_ms), 5),
                               "propagates_per_s": round(1e3 / statistics.fmean(flush_ms), 1),
                               "note": "320 MiB write before each step instead of rotation"},
             "rel_l2_vs_fp64_oracle": err, "energy_err": eerr}

    # ------------------------------------------------------------ variants --
    if rank == 0 and not args.quick:
        ranks_in_step["on"] = False  # only rank 0 runs this section
        ks = max(10, min(200, args.steps // 10))
        specs = [B.fft2(fi) for fi, _ in slots]
        with clocks.window():
            st_ms, _ = timed(lambda i: spec_state(n, specs[i % R], slots[i % R][1]), ks, 3)
            _, st_pass = timed(lambda i: spec_state(n, specs[i % R], slots[i % R][1]), ks, 3, 2)
            pl, _ = timed(lambda i: plain(n, *slots[i % R]), ks, 3)
            pl64, _ = timed(lambda i: plain(n, *slots[i % R], fp64=True), max(5, ks // 4), 3)
            # external reference point: cuFFT (torch.fft) fft2 -> H grid multiply -> ifft2
            Hc = torch.polar(torch.ones(n, n, device=dev, dtype=torch.float64),
                             torch.as_tensor(-2 * np.pi * np.mod(g["Kz"] * Z, 1.0),
                                             device=dev)).to(torch.complex64)

            def cufft_plain(i):
                fi, fo = slots[i % R]
                fo.copy_(torch.fft.ifft2(torch.fft.fft2(fi) * Hc))
                return 0
            cu, _ = timed(cufft_plain, ks, 3)
            del Hc
            # the reference's own sequence on the GPU (what its CuPy path runs):
            # cuFFT fft2, H = exp(2*pi*i*(trunc(Kz z) - Kz z)) built in FP64 from a
            # cached FP64 Kz grid every call (beam2d.py:485-489), multiply, ifft2
            Kz_d = torch.as_tensor(g["Kz"], device=dev)

            def cufft_fp64h(i):
                fi, fo = slots[i % R]
                dk = Kz_d * Z
                h = torch.polar(torch.ones_like(dk), 2 * np.pi * (torch.trunc(dk) - dk))
                fo.copy_(torch.fft.ifft2(torch.fft.fft2(fi) * h.to(torch.complex64)))
                return 0
            cu64, _ = timed(cufft_fp64h, max(5, ks // 4), 3)
            del Kz_d
        del specs
        torch.cuda.synchronize()
        # FP32-phase vs float-float phase error at every z of the workload
        f0 = O.gaussian(n, AREA, 1.0, WAIST)
        s0 = torch.as_tensor(np.fft.fft2(f0).astype(np.complex64), device=dev)
        zerr = {}
        for z in (0.1, 1.0, 5.0, 10.0, 50.0):
            _, fr = O.propagate(np.fft.fft2(f0), g["Kz"], z)
            a = B.propagate(s0, AREA, WL, z, write_spectrum=False)
            b = B.propagate(s0, AREA, WL, z, write_spectrum=False, flags=L.LP_FLAG_PHASE_FP32)
            torch.cuda.synchronize()
            ah, bh = a.cpu().numpy(), b.cpu().numpy()
            zerr[str(z)] = {"ff_phase": O.rel_l2(ah, fr), "fp32_phase": O.rel_l2(bh, fr),
                            "ff_phase_energy_err": O.energy_err(ah, fr),
                            "fp32_phase_energy_err": O.energy_err(bh, fr)}
        sweep = {}
        for nn in (512, 1024, 2048, 4096):
            rr = nslots(nn)
            sl = make(nn, rr)
            with clocks.window():
                sm, _ = timed(lambda i: fused(nn, *sl[i % rr]), ks, 3)
            ms = statistics.fmean(sm)
            sweep[str(nn)] = {"ms": round(ms, 5), "propagates_per_s": round(1e3 / ms, 1),
                              "effective_gbs": round(16 * nn * nn / (ms * 1e-3) / 1e9, 1)}
            del sl
        # complex128 (complex_bits=128, the reference's default dtype): the
        # complex128 family (float-float transforms) on the same workload
        z128_in = torch.as_tensor(O.gaussian(n, AREA, 1.0, WAIST).astype(np.complex128),
                                  device=dev)
        z128_out = torch.empty_like(z128_in)

        def c128_step(i):
            # the tensor wrapper checks dtype and shape before the ABI call
            B.propagate_field(z128_in, AREA, WL, Z, out=z128_out)
            return 0
        with clocks.window():
            zms, _ = timed(c128_step, 10, 3)
        _, z_ref = O.propagate(np.fft.fft2(O.gaussian(n, AREA, 1.0, WAIST)), g["Kz"], Z)
        torch.cuda.synchronize()
        extra["complex128_propagate"] = {
            "ms": round(statistics.fmean(zms), 4),
            "rel_l2_vs_fp64_oracle": O.rel_l2(z128_out.cpu().numpy(), z_ref),
            "note": "lp_propagate_field_c128: float-float transforms on the FP32 pipes, "
                    "the reference's float64 Kz and phase"}
        del z128_in, z128_out
        st = statistics.fmean(st_ms)
        extra.update({
            "spectrum_state_propagate": {
                "ms": round(st, 5), "propagates_per_s": round(1e3 / st, 1),
                "effective_gbs": round(16 * n * n / (st * 1e-3) / 1e9, 1),
                "passes_ms": [round(statistics.fmean(p), 5) for p in st_pass]},
            "plain_unfused": {"ms": round(statistics.fmean(pl), 5),
                              "propagates_per_s": round(1e3 / statistics.fmean(pl), 1),
                              "fused_speedup": round(statistics.fmean(pl) / ms_step, 3)},
            "plain_unfused_fp64_h": {"ms": round(statistics.fmean(pl64), 5),
                                     "fused_speedup": round(statistics.fmean(pl64) / ms_step, 3)},
            "cufft_fp64_h_reference_sequence": {
                "ms": round(statistics.fmean(cu64), 5),
                "fused_speedup": round(statistics.fmean(cu64) / ms_step, 3),
                "note": "the reference's propagate sequence on the GPU: torch.fft fft2, FP64 H "
                        "from a cached FP64 Kz grid every call, multiply, ifft2; not part of "
                        "the product"},
            "cufft_plain_reference_point": {
                "ms": round(statistics.fmean(cu), 5),
                "fused_speedup": round(statistics.fmean(cu) / ms_step, 3),
                "note": "torch.fft (cuFFT) fft2, H grid multiply, ifft2; not part of the product"},
            "phase_error_by_z": zerr, "sweep": sweep})

        # Differentiable phase-mask design: 1024^2, 1 mm, 1064 nm, waist 300 um,
        # z = 10 cm, 16 Gaussian spots (waist 20 um), 200 Adam steps.
        from lightprop2d_gb300 import autograd as A
        from lightprop2d_gb300 import design as D
        torch.cuda.synchronize()
        dargs = dict(n=1024, area=0.1, wl=1064e-7, waist=300e-4, z=10.0, steps=200, lr=0.05,
                     seed=0)
        te, tg = {}, {}
        t0 = time.perf_counter()
        with clocks.window():
            _, losses = D.design_phase_mask(**dargs, timing=te)
        torch.cuda.synchronize()
        t_design = time.perf_counter() - t0
        with clocks.window():
            _, losses_g = D.design_phase_mask(**dargs, graph=True, timing=tg)
        extra["inverse_design"] = {
            "grid": 1024, "adam_steps": 200,
            "ms_per_step_graph": round(tg["ms_per_step"], 4),
            "ms_per_step_eager": round(te["ms_per_step"], 4),
            "wall_s_eager_incl_setup": round(t_design, 3),
            "loss_first": losses[0], "loss_last": losses[-1], "loss_last_graph": losses_g[-1],
            "note": "forward fused kernel + adjoint kernel + loss + Adam per step; graph = "
                    "the whole step captured in a CUDA graph and replayed"}

        # Split-step chain: 4096^2, 5 mm, 1550 nm, 64 x [propagate(5 cm), screen],
        # Gaussian screens (corr 200 um, RMS 1 rad), checkpoint every 8 steps.
        nn, K = 4096, 64
        screens = D.gaussian_screens(K, nn, 0.5, corr_len=200e-4, rms=1.0, seed=1)
        u0 = D.gaussian_field(nn, 0.5, 0.1)
        sc = screens.clone().requires_grad_(True)
        torch.cuda.synchronize()
        base = torch.cuda.memory_allocated()
        torch.cuda.reset_peak_memory_stats()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        with clocks.window():
            ev[0].record(stream)
            y = A.split_step_chain(u0, sc, 5.0, 0.5, 1550e-7, checkpoint_every=8)
            ev[1].record(stream)
            (y.real ** 2 + y.imag ** 2).sum().backward()
            ev[2].record(stream)
            torch.cuda.synchronize()
        extra["split_step_chain"] = {
            "grid": nn, "steps": K, "checkpoint_every": 8,
            "forward_ms": round(ev[0].elapsed_time(ev[1]), 3),
            "backward_ms": round(ev[1].elapsed_time(ev[2]), 3),
            "peak_extra_gib": round((torch.cuda.max_memory_allocated() - base) / 2 ** 30, 3),
            "screens_gib": round(screens.numel() * 4 / 2 ** 30, 3)}
        del screens, sc, y, u0
        torch.cuda.empty_cache()

        # Uneven batch: 4096 beams in one persistent launch (CUDA graph).
        if world == 1:
            extra["batch_uneven"] = batch_section(dev, stream, clocks, reps=20)
            torch.cuda.empty_cache()

        # Metrics, generators, grid management, mode decomposition.
        with clocks.window():
            extra["next_rows"] = next_rows_section(dev, stream, hbm)
        torch.cuda.empty_cache()

    # ------------------------------------------ uneven batch, sharded (N > 1) --
    # Every rank runs its share of the 4096 beams (batch.shard: points
    # balanced, no collective on the data path) as one graph-replayed launch;
    # the batch takes as long as the slowest rank.
    if world > 1 and not args.quick:
        ranks_in_step["on"] = True
        dist.barrier()
        mine = batch_section(dev, stream, clocks, reps=20, check_oracle=(rank == 0),
                             compare=False, shard_of=(world, rank))
        per = [None] * world
        dist.all_gather_object(per, {"rank": rank, **mine})
        t_max = max(r["ms_per_batch"] for r in per)
        nb_all = sum(r["beams"] for r in per)
        extra["batch_uneven"] = {
            "workload": "4096 beams: " + ", ".join(f"{c} x {n}^2" for n, c in BATCH_MIX)
                        + ", hole+lens+propagate+iprofile, wl 632 nm; sharded over ranks",
            "ranks": world, "beams": nb_all, "ms_per_batch": round(t_max, 4),
            "beams_per_s": round(nb_all / (t_max * 1e-3), 1),
            "points_per_s": round(sum(r["points"] for r in per) / (t_max * 1e-3), 1),
            "per_rank": [{k: r[k] for k in ("rank", "beams", "points", "ms_per_batch")}
                         for r in per],
            "rel_l2_vs_fp64_oracle_rank0": per[0]["rel_l2_vs_fp64_oracle"],
            "energy_rel_err_max": max(r["energy_rel_err_max_all_beams"] for r in per)}
        torch.cuda.empty_cache()

    # ----------------------------------------------------------------- e2e --
    # Each step: pinned host -> device copy of the field, the fused
    # propagate through the C ABI, device -> pinned host copy of the result.
    # Steps are pipelined over three streams (copy in, compute, copy out) and
    # three device/host slot sets, so step i+1's upload and step i-1's
    # download overlap step i's propagate, as a streaming user would run it.
    hin = torch.empty((n, n), dtype=torch.complex64, pin_memory=True)
    hin.copy_(torch.as_tensor(O.gaussian(n, AREA, 1.0, WAIST).astype(np.complex64)))
    RE = 3
    houts = [torch.empty((n, n), dtype=torch.complex64, pin_memory=True) for _ in range(RE)]
    dins = [torch.empty((n, n), dtype=torch.complex64, device=dev) for _ in range(RE)]
    douts = [torch.empty((n, n), dtype=torch.complex64, device=dev) for _ in range(RE)]
    s_in, s_cmp, s_out = (torch.cuda.Stream(device=dev) for _ in range(3))
    sp_cmp = ctypes.c_void_p(s_cmp.cuda_stream)
    ev_in = [torch.cuda.Event() for _ in range(RE)]
    ev_cmp = [torch.cuda.Event() for _ in range(RE)]
    ev_out = [torch.cuda.Event() for _ in range(RE)]

    def e2e_step(i):
        k = i % RE
        s_in.wait_event(ev_cmp[k])             # slot's previous propagate has read dins[k]
        with torch.cuda.stream(s_in):
            dins[k].copy_(hin, non_blocking=True)
        ev_in[k].record(s_in)
        s_cmp.wait_event(ev_in[k])
        s_cmp.wait_event(ev_out[k])            # douts[k] downloaded already
        L.check(lib.lp_propagate_field(vp(dins[k]), vp(douts[k]), nul, nul, n, AREA, WL, Z,
                                       0.0, nul, 0, nul, 0, 0, sp_cmp), "e2e step")
        ev_cmp[k].record(s_cmp)
        s_out.wait_event(ev_cmp[k])
        with torch.cuda.stream(s_out):
            houts[k].copy_(douts[k], non_blocking=True)
        ev_out[k].record(s_out)

    ke = max(10, min(200, args.steps // 10))
    if dist:
        dist.barrier()  # every rank streams at once (rank 0 may come from its own section)
    with clocks.window():
        for i in range(3 * RE):
            e2e_step(i)
        torch.cuda.synchronize()
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea.record(s_in)
        for i in range(ke):
            e2e_step(i)
        eb.record(s_out)
        torch.cuda.synchronize()
    e2e_t = ea.elapsed_time(eb) / ke
    if dist:
        t = torch.tensor([e2e_t], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t)
    e2e_err = O.rel_l2(houts[(ke - 1) % RE].numpy(), f_ref)

    # The host link bounds a step: the same uploads and downloads without
    # the propagate (both directions at once, as in the pipeline), and each
    # direction alone.
    def link_time(do_in, do_out):
        def once(i):
            k = i % RE
            if do_in:
                with torch.cuda.stream(s_in):
                    dins[k].copy_(hin, non_blocking=True)
            if do_out:
                with torch.cuda.stream(s_out):
                    houts[k].copy_(douts[k], non_blocking=True)
        for i in range(RE):
            once(i)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s_in)
        s_out.wait_event(a)
        for i in range(ke):
            once(i)
        s_in.wait_stream(s_out)
        b.record(s_in)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / ke

    link_both = link_time(True, True)
    link_in, link_out = link_time(True, False), link_time(False, True)
    link = {"ms_per_step_copies_only": round(link_both, 5),
            "h2d_gbs": round(8 * n * n / link_in / 1e6, 1),
            "d2h_gbs": round(8 * n * n / link_out / 1e6, 1),
            "both_gbs_per_direction": round(8 * n * n / link_both / 1e6, 1),
            "e2e_frac_of_link_bound": round(link_both / e2e_t, 4)}

    # ------------------------------------------------------ e2e: Beam2D --
    # The reference user's loop (tests/hole_diffraction.py:37-42 of the
    # reference): one Beam2D built from a host field, then per step
    # propagate(dz) and the iprofile read back to numpy.  Host wall clock
    # around the steps (each iprofile read synchronises).
    beam2d_e2e = None
    if rank == 0:
        from lightprop2d_gb300 import Beam2D
        f_host = O.gaussian(n, AREA, 1.0, WAIST).astype(np.complex64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bm = Beam2D(AREA, n, WL, init_field=f_host, complex_bits=64)
        _ = bm.iprofile
        t_ctor = time.perf_counter() - t0
        kb = max(10, min(100, args.steps))
        with clocks.window():
            for _ in range(3):
                bm.propagate(Z)
                _ = bm.iprofile
            t0 = time.perf_counter()
            for _ in range(kb):
                bm.propagate(Z)
                ip = bm.iprofile
            t_b2d = (time.perf_counter() - t0) / kb
        o = O.OracleBeam(AREA, n, WL, init_field=O.gaussian(n, AREA, 1.0, WAIST))
        o.propagate(Z * (kb + 3))
        ip_ref = np.abs(o.field) ** 2
        # the same loop with Beam2D's default complex_bits=128 (the dtype the
        # reference's own scripts run in): float-float transforms, float64
        # iprofile (32 MiB read back per step)
        bz = Beam2D(AREA, n, WL, init_field=O.gaussian(n, AREA, 1.0, WAIST))
        kz = max(5, min(40, args.steps))
        with clocks.window():
            for _ in range(2):
                bz.propagate(Z)
                _ = bz.iprofile
            t0 = time.perf_counter()
            for _ in range(kz):
                bz.propagate(Z)
                ipz = bz.iprofile
            t_z = (time.perf_counter() - t0) / kz
        # Beam2D's first propagate is the fused field -> field call, which
        # stores spectrum * H(Z); later ones apply H(sum of the rest) to it:
        # the oracle takes the same two steps (at ~40 cm one ulp of Kz*z is
        # ~1e-10 of phase, so one H(42 Z) would differ by that much)
        oz = O.OracleBeam(AREA, n, WL, init_field=O.gaussian(n, AREA, 1.0, WAIST))
        oz.propagate(Z)
        oz.propagate(Z * (kz + 1))
        ipz_ref = np.abs(oz.field) ** 2
        beam2d_c128 = {
            "value": 1.0 / t_z, "unit": UNIT, "ms_per_step": round(t_z * 1e3, 4),
            "d2h_bytes_per_step": 8 * n * n, "dtype": "c128 (float-float transforms)",
            "iprofile_rel_l2_vs_fp64_oracle": float(np.linalg.norm(ipz - ipz_ref) /
                                                    np.linalg.norm(ipz_ref)),
            "note": "the e2e_beam2d loop with complex_bits=128 (Beam2D's default)"}
        beam2d_e2e = {
            "value": 1.0 / t_b2d, "unit": UNIT, "ms_per_step": round(t_b2d * 1e3, 4),
            "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 4 * n * n,
            "construct_ms_incl_h2d": round(t_ctor * 1e3, 3),
            "iprofile_rel_l2_vs_fp64_oracle": float(np.linalg.norm(ip - ip_ref) /
                                                    np.linalg.norm(ip_ref)),
            "note": "Beam2D(init_field=host array), then per step propagate(1 cm) and "
                    "iprofile to numpy (the reference user's loop); host wall clock",
            "complex_bits_128": beam2d_c128}
    clocks.stop()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64", "data": "synthetic",
            "config": bench_config(),
            "l2_rotation": f"{R} in/out grid pairs ({R * 16 * n * n / 2**20:.0f} MiB)",
            "parallelism": f"replicas{world}",
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": round(achieved, 1),
                         "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4),
                         "traffic": NCU_DRAM_BYTES_2048.get(names[dom]) if n == 2048 else None,
                         "traffic_note": "ncu dram__bytes_read+write per launch, warm L2",
                         "step_dram_bytes_ncu": sum(NCU_DRAM_BYTES_2048.values()),
                         "ncu_pipes": NCU_PIPES_2048.get(names[dom]) if n == 2048 else None,
                         "alg_bytes_per_launch": alg_bytes},
            "cpu_baseline": cb,
            "e2e": {"value": world * 1e3 / e2e_t, "unit": UNIT,
                    "h2d_bytes_per_step": 8 * n * n, "d2h_bytes_per_step": 8 * n * n,
                    "ms_per_step": round(e2e_t, 5), "rel_l2_vs_fp64_oracle": e2e_err,
                    "host_link": link,
                    "note": "pinned H2D, propagate, D2H per step; three-stream pipeline; "
                            "host_link: the same copies without the propagate"},
            "e2e_beam2d": beam2d_e2e,
            "clocks": clocks.summary(),
            "gpu_launches": 3 * args.steps,
            **extra,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
