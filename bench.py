#!/usr/bin/env python3
"""Benchmark of the GB300 DPM step (one JSON line on stdout).

Headline workload, the batched 2D sweep: 512 independent tissues with
N ~ U{8..256} cells and NV ~ {16, 24, 32, 48} vertices per cell (one NV per
tissue), per-tissue kb ~ LogU[1e-3, 1e-1], calA0 ~ U[1.0, 1.3], true packing
fraction ~ U[0.6, 0.9] (phi0 = sqrt(phi)), ka = kl = kc = 1, r0 = 1,
dt = 0.005.  Cells start as the Cell2D constructor's regular polygons, centred
on a seeded, jittered square lattice of the tissue's periodic box (synthetic
data; the reference names no dataset).  All tissues step together in one
batch; each simulation step is one launch of the fused step kernel, and the
neighbour-list rebuild plus one rebuild period of steps (chosen with warps
per block and the kernel variant by the project's autotuner,
dpm2d_autotune) are one captured CUDA graph.

One benchmark "step" is one dpm2d_step call of 32 simulation steps of the
whole batch.  L2 (129 MB) is flushed by writing 256 MB before every timed
iteration, outside the timed events.  value = vertices * simulation steps /
time.

Also reported (keys of the same line): the plain single-system paths -- the
1,024-cell compression protocol ("plain"), the 16-cell run of 10,000 steps
("plain_c0"), the 256-cell 3D monolayer ("plain3d", and "plain3d_sub2" at
the reference's own 162-vertex mesh) -- the sweep's own
tissues run one after another through the plain path ("sequential"; the
same for the 3D batch and for the served requests), 48 monolayers in one
batch ("batched3d"), the same 32-tissue sample the reference arm times
("same_sample"), the sweep's full 20,000-step run ("steady_state"), the
reference's dispersion on the device ("disperse"), the dominant kernel's HBM
and issue rooflines, the end-to-end rate through the C ABI with pinned host
buffers ("e2e"), the served mixed stream of 2D and 3D requests through
dpm_serve_* with p50/p99 latency ("served"), SM clocks during the timed
region, and CPU baselines (the oracle restatement of the reference on the
host cores, single-thread and all-core).

The GPU arm builds its inputs with the product's own host model (clDPM); the
reference arm (--impl reference) builds the same inputs with the oracle and
never imports the product.  Both builders give the same bits
(tests/test_bench_workloads.py).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--serve-requests R] [--cpu-budget S]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vertex-steps/s batched+served vs plain on 1 GB300; p50/p99 run latency; HBM GB/s"
UNIT = "vertex-steps/s"
DT = 0.005
SIM_STEPS = 32  # simulation steps per benchmark step (a multiple of every rebuild period)
SWEEP_SEED = 1000
SAMPLE_EVERY = 16  # the CPU sample: every 16th tissue of the sweep
L2_FLUSH_BYTES = 256 << 20
WORKLOAD_SWEEP = ("batched 2D sweep: 512 tissues, N~U{8..256}, NV in {16,24,32,48}, "
                  "kb~LogU[1e-3,1e-1], calA0~U[1,1.3], phi~U[0.6,0.9], ka=kl=kc=1, r0=1, dt=0.005")
L2_NOTE = "256 MB written before every timed iteration of the GPU arm (outside the events)"


# ---------------------------------------------------------------------------
# geometry providers
# ---------------------------------------------------------------------------

class ProductGeometry:
    """Cells and boxes from the product's host model (clDPM): the GPU arm."""

    def __init__(self):
        from opencl_dpm_gb300 import clDPM
        self.m = clDPM

    def tissue2d(self, calA, nv, r0, phi0):
        """Regular polygons at the origin, their rest area and edge, and the
        box of the Tissue2D constructor (L = sqrt(sum A) / phi0)."""
        proto = [self.m.Cell2D(0.0, 0.0, float(calA[i]), int(nv[i]), float(r0[i]))
                 for i in range(len(nv))]
        L = self.m.Tissue2D(proto, float(phi0)).L
        return ([np.asarray(p.Verts, np.float32) for p in proto],
                np.float32([p.a0 for p in proto]), np.float32([p.l0 for p in proto]),
                np.float32(L))


class OracleGeometry:
    """The same from the oracle (oracle/): the reference arm, which must not
    load the product."""

    def __init__(self):
        from oracle.oracle import Port
        self.P = Port()

    def tissue2d(self, calA, nv, r0, phi0):
        xs, a0, l0, areas = [], [], [], []
        for i in range(len(nv)):
            xy, a, l, _ = self.P.cell2d(0.0, 0.0, float(calA[i]), int(nv[i]), float(r0[i]))
            xs.append(xy)
            a0.append(a)
            l0.append(l)
            areas.append(self.P.area2d(xy))
        return xs, np.float32(a0), np.float32(l0), np.float32(self.P.box2d(areas, float(phi0)))


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def lattice_centres(rng, n, L, jitter=0.1):
    m = int(math.ceil(math.sqrt(n)))
    sp = L / m
    sites = rng.permutation(m * m)[:n]
    ix, iy = sites % m, sites // m
    c = np.stack([(ix + 0.5) * sp, (iy + 0.5) * sp], axis=1)
    c += rng.uniform(-jitter * sp, jitter * sp, size=c.shape)
    return c.astype(np.float32)


def build_tissue(geo, rng, n, nv, calA, r0, Kb, phi, centres="lattice"):
    """One tissue: regular polygons at jittered lattice (or uniform) centres."""
    polys, a0, l0, L = geo.tissue2d(calA, nv, r0, np.sqrt(phi))
    if centres == "lattice":
        cen = lattice_centres(rng, n, L)
    else:
        cen = rng.uniform(0.0, L, size=(n, 2)).astype(np.float32)
    xy = np.concatenate([polys[i] + cen[i] for i in range(n)])
    return dict(nv=np.asarray(nv, np.uint32), xy=xy, a0=a0, l0=l0,
                r0=np.asarray(r0, np.float32), Ka=np.ones(n, np.float32),
                Kl=np.ones(n, np.float32), Kb=np.full(n, Kb, np.float32), L=L, Kre=1.0,
                Kat=0.0)


def workload_batched(geo, seed=SWEEP_SEED, ntissues=512):
    rng = np.random.default_rng(seed)
    tissues = []
    for _ in range(ntissues):
        n = int(rng.integers(8, 257))
        nv = int(rng.choice([16, 24, 32, 48]))
        kb = float(10 ** rng.uniform(-3, -1))
        calA = rng.uniform(1.0, 1.3, n)
        phi = float(rng.uniform(0.6, 0.9))
        tissues.append(build_tissue(geo, rng, n, np.full(n, nv), calA, np.ones(n), kb, phi))
    return tissues


def workload_c1(geo, seed=1, n=1024):
    """1,024 cells x 32 vertices, bidisperse r0 1.0 / 1.4 (shuffled), calA0 ~
    U[1, 1.2], kb = 0.01, at true packing fraction 0.6."""
    rng = np.random.default_rng(seed)
    r0 = rng.permutation(np.r_[np.full(n // 2, 1.0), np.full(n - n // 2, 1.4)])
    calA = rng.uniform(1.0, 1.2, n)
    return [build_tissue(geo, rng, n, np.full(n, 32), calA, r0, 0.01, 0.6)]


def workload_c0(geo, seed=2):
    """16 cells x 32 vertices, calA0 = 1, kb = 0, uniform random centres at
    true packing fraction 0.6."""
    rng = np.random.default_rng(seed)
    return [build_tissue(geo, rng, 16, np.full(16, 32), np.ones(16), np.ones(16), 0.0, 0.6,
                         centres="uniform")]


def sweep_sample(tissues):
    return tissues[::SAMPLE_EVERY]


def sample_desc(tissues):
    s = sweep_sample(tissues)
    return (f"{len(s)} of {len(tissues)} tissues (every {SAMPLE_EVERY}th, "
            f"{sum(int(t['nv'].sum()) for t in s)} vertices)")


DT3 = 0.002  # 3D monolayer time step


def build_monolayer(clDPM, rng, n, level, r0=1.0):
    """n icospheres (Cell3D ctor geometry) resting on z = 0, centres on a
    jittered hexagonal lattice (spacing 2 r0, jitter U[-0.1, 0.1]) in a
    periodic box; kv=1, ka=0.5, ks=0.1, kb=0.05, adhesion range 0.1.  Target
    volume 1.0x the initial mesh volume; target area 1.05x the initial true
    mesh area (the constructor's SurfaceArea is twice the area), spread over
    the faces, with the rest edge from it by the reference's rule
    l0 = sqrt(4 a0) / sqrt(3)."""
    proto = clDPM.Cell3D([0.0, 0.0, 0.0], 1.0, r0, level)
    ring = np.asarray(proto.Verts, np.float32)
    faces = np.asarray(proto.GetFaces(), np.uint32)
    m = int(math.ceil(math.sqrt(n)))
    sp = 2.0 * r0
    L = np.float32(m * sp)
    sites = rng.permutation(m * m)[:n]
    ix, iy = sites % m, sites // m
    cx = ((ix + 0.5 + 0.5 * (iy % 2)) * sp) % L + rng.uniform(-0.1, 0.1, n)
    cy = (iy + 0.5) * sp + rng.uniform(-0.1, 0.1, n)
    cen = np.stack([cx, cy, np.full(n, r0)], axis=1).astype(np.float32)
    xyz = np.concatenate([ring + cen[i] for i in range(n)])
    v0 = np.float32(proto.Volume)
    a_face = np.float32(1.05 * (0.5 * float(proto.SurfaceArea)) / int(proto.NF))
    a0 = np.full(n, a_face, np.float32)
    # the host model's rest edge: sqrt(double(4 a0)) / sqrt(3), 4 a0 in float
    l0 = (np.sqrt((np.float32(4.0) * a0).astype(np.float64)) / np.sqrt(3.0)).astype(np.float32)
    f = lambda v: np.full(n, v, np.float32)
    return dict(dim=3, nv=int(proto.NV), faces=faces, xyz=xyz, Kv=f(1.0), Ka=f(0.5), Ks=f(0.1),
                v0=f(v0), a0=a0, l0=l0, Kb=f(0.05), adh=f(0.1), L=L, Kre=1.0, level=level)


C2_NOTE = ("kv=1 ka=0.5 ks=0.1 kb=0.05, adhesion range 0.1, v0 = initial mesh volume, "
           "target area 1.05x the initial mesh area, dt=0.002")


def make_batch(ctx, tissues):
    from opencl_dpm_gb300.abi import Batch2D
    cat = lambda k: np.concatenate([t[k] for t in tissues])
    b = Batch2D(ctx, [len(t["nv"]) for t in tissues], cat("nv"))
    b.set_cells(cat("Ka"), cat("Kl"), cat("Kb"), cat("a0"), cat("l0"), cat("r0"))
    b.set_tissues([t["L"] for t in tissues], [t["Kre"] for t in tissues],
                  [t["Kat"] for t in tissues], 1)
    xy = cat("xy")
    b.upload(xy)
    return b, xy


def make_batch3d(ctx, ts):
    from opencl_dpm_gb300.abi import Batch3D
    cat = lambda k: np.concatenate([t[k] for t in ts])
    b = Batch3D(ctx, [len(t["Kv"]) for t in ts], ts[0]["faces"], ts[0]["nv"])
    b.set_cells(cat("Kv"), cat("Ka"), cat("Ks"), cat("v0"), cat("a0"), cat("l0"), cat("Kb"),
                cat("adh"))
    b.set_tissues([t["L"] for t in ts], 1.0, 1)
    b.upload(cat("xyz"))
    return b


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during timing."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            v = json.load(f)["hbm_gbs"]
        return float(v), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_rows(summary):
    """Rows of the committed ncu summary `profiles/<summary>.md`: the
    'traffic (read + write) per launch' and 'warp instructions per launch'
    figures and the build the capture was taken of."""
    p = os.path.join(ROOT, "profiles", summary + ".md")
    out = {"traffic": None, "warp_inst": None, "build": None}
    units = {"MB": 1e6, "GB": 1e9, "KB": 1e3, "M": 1e6, "G": 1e9, "k": 1e3}
    try:
        with open(p) as f:
            for line in f:
                cells = [c.strip() for c in line.split("|")]
                if len(cells) < 3:
                    continue
                key = cells[1]
                try:
                    if key.startswith("traffic (read + write) per launch"):
                        v, unit = cells[2].split()[:2]
                        out["traffic"] = float(v) * units[unit]
                    elif key.startswith("warp instructions per launch"):
                        v, unit = cells[2].split()[:2]
                        out["warp_inst"] = float(v) * units[unit]
                    elif key.startswith("build captured"):
                        out["build"] = cells[2]
                except (ValueError, KeyError):
                    pass
    except OSError:
        pass
    return out


def slot_classes(tissues):
    """Vertex-slot classes of a batch (one step launch each): the class of a
    tissue is that of its largest ring (<= 32, 64, 128, 256 vertices)."""
    return len({min(3, max(0, math.ceil(math.log2(int(t["nv"].max()) / 32))))
                for t in tissues})


def launches_per_call(batch, tissues, sim_steps, period):
    """Kernel launches of one dpm2d_step(sim_steps): per rebuild period one
    bin-preparation launch, 3 launches per radix pass, one neighbour-list
    launch; per simulation step one fused step launch per vertex-slot
    class."""
    lb, _, _, _ = batch.bins()
    tbits = int(math.ceil(math.log2(batch.ntissues))) if batch.ntissues > 1 else 0
    passes = (lb + tbits + 7) // 8
    blocks = math.ceil(sim_steps / period)
    return blocks * (1 + 3 * passes + 1) + sim_steps * slot_classes(tissues)


def reduce_over_ranks(secs, units, world, device):
    """Whole-job timing of independent shards: the slowest rank's time and
    the units of all ranks (one all-reduce each, outside the timed region;
    the shards exchange nothing while stepping)."""
    if world <= 1:
        return secs, units
    import torch
    import torch.distributed as dist
    t = torch.tensor([secs], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.barrier()
    return float(t.item()), float(u.item())


class Timer:
    """CUDA-event timing on the context's stream, L2 flushed before each
    iteration (outside the events)."""

    def __init__(self, ctx, device):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
        self.flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32,
                                 device=f"cuda:{device}")

    def __call__(self, iters, fn, flush=True):
        """Seconds per iteration (mean)."""
        torch = self.torch
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(iters)]
        with torch.cuda.stream(self.stream):
            for i in range(iters):
                if flush:
                    self.flush.zero_()
                ev[i][0].record(self.stream)
                fn()
                ev[i][1].record(self.stream)
        torch.cuda.synchronize()
        self.ctx.synchronize()
        return sum(s.elapsed_time(e) for s, e in ev) / iters / 1e3

    def span(self, fn):
        """Seconds of fn() between two events on the stream (fn may
        synchronize the stream itself)."""
        torch = self.torch
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(self.stream):
            a.record(self.stream)
            out = fn()
            b.record(self.stream)
        torch.cuda.synchronize()
        self.ctx.synchronize()
        return a.elapsed_time(b) / 1e3, out


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args, rank, world, local_rank):
    import torch
    from opencl_dpm_gb300.abi import Context

    torch.cuda.set_device(local_rank)
    ctx = Context(local_rank)
    timed = Timer(ctx, local_rank)
    geo = ProductGeometry()

    tissues = workload_batched(geo, seed=SWEEP_SEED + rank)
    b, xy_host = make_batch(ctx, tissues)
    V, N = b.nverts, b.ncells
    tuned = b.autotune(DT, trial_blocks=2, use_cache=True)

    for _ in range(max(3, args.warmup)):
        b.step(SIM_STEPS, DT)
    ctx.synchronize()

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    torch.cuda.nvtx.range_push("headline")
    secs = timed(args.steps, lambda: b.step(SIM_STEPS, DT)) * args.steps
    torch.cuda.nvtx.range_pop()
    clock_info = clocks.stop()
    torch.cuda.synchronize()
    secs, units = reduce_over_ranks(secs, float(V) * SIM_STEPS * args.steps, world,
                                    f"cuda:{local_rank}")
    value = units / secs
    ms_per_step = secs / args.steps * 1e3

    if rank != 0:
        return None

    roofline = step_roofline(b, timed, V, N, ms_per_step, tuned, clock_info)
    e2e = e2e_leg(b, timed, V, args)
    sample = same_sample_leg(ctx, timed, tissues, args)

    c1 = plain_c1(ctx, timed, geo)
    c0 = plain_c0(ctx, timed, geo)
    p3 = plain3d(ctx, timed, max(3, args.steps))
    p3s2 = plain3d(ctx, timed, max(3, args.steps), level=2)
    b3 = batched3d(ctx, timed, max(3, args.steps))
    b3["batched_over_plain"] = round(b3["value"] / p3["value"], 2)
    seq2 = sequential_2d(ctx, timed, tissues)
    seq3 = sequential_3d(ctx, timed, workload_batched3d())
    b3["sequential"] = seq3
    b3["batched_over_sequential"] = round(b3["value"] / seq3["value"], 2)
    steady = steady_state_leg(ctx, timed, geo)
    disp = disperse_leg(ctx, tissues, geo)

    served = None
    if args.serve_requests > 0:
        served = run_served(ctx, timed, args.serve_requests, plain2d=c1["value"],
                            plain3d=p3["value"])

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded tissues; see config)",
        "config": sweep_config(b.ntissues, N, V),
        "graph": "one CUDA graph replay per cell-list rebuild period",
        "tuning": tuned,
        "gpu_launches": launches_per_call(b, tissues, SIM_STEPS,
                                          tuned["rebuild_period"]) * args.steps,
        "roofline": roofline, "e2e": e2e, "same_sample": sample,
        "plain": c1,
        "batched_over_plain": round(value / world / c1["value"], 2),
        "sequential": seq2,
        "batched_over_sequential": round(value / world / seq2["value"], 2),
        "plain_c0": c0,
        "plain3d": p3,
        "plain3d_sub2": p3s2,
        "batched3d": b3,
        "steady_state": steady,
        "disperse": disp,
        "served": served,
        "clocks": clock_info,
    }
    line["cpu_baseline"] = cpu_baseline(tissues, budget_s=args.cpu_budget)
    line["cpu_baselines"] = cpu_baselines_plain(geo, args.cpu_budget)
    return line


def sweep_config(ntissues, ncells, nverts):
    """The workload both arms name (identical on both)."""
    return {"workload": WORKLOAD_SWEEP, "tissues": ntissues, "cells": ncells,
            "vertices": nverts, "seed": SWEEP_SEED, "sim_steps_per_step": SIM_STEPS,
            "l2": L2_NOTE}


def step_roofline(b, timed, V, N, ms_per_step, tuned, clock_info):
    """HBM and issue rooflines of the fused step kernel (k2d_step)."""
    # one launch at a time after an L2 flush (cold); one rebuild period of
    # step launches queued back to back after a fresh neighbour-list rebuild
    # (warm, without the graph: each launch forks the vertex-slot classes
    # over two streams by events); and the step launches' share of the graph
    # replays: the same call timed (L2 flushed, as the headline) at the tuned
    # rebuild period and at half of it, whose difference is the extra
    # rebuilds inside the graph; the headline call less its rebuilds is the
    # step launches' time
    nk = 20
    kern = timed(nk, lambda: b.step_kernel(DT))
    period = tuned["rebuild_period"]

    def period_of_steps():
        for _ in range(period):
            b.step_kernel(DT)

    b.rebuild_now()
    back_to_back = timed(1, period_of_steps, flush=False) / period
    call = lambda: b.step(SIM_STEPS, DT)
    rebuild, in_graph, t_full = None, back_to_back, None
    if period % 4 == 0 and SIM_STEPS % period == 0:
        t_full = timed(10, call)
        b.set_tuning(rebuild_period=period // 2)
        call()  # captures the graph of the shorter period
        t_half = timed(10, call)
        b.set_tuning(rebuild_period=period)
        call()
        n_full, n_half = SIM_STEPS // period, SIM_STEPS // (period // 2)
        rebuild = (t_half - t_full) / (n_half - n_full)
        in_graph = (ms_per_step / 1e3 - n_full * rebuild) / SIM_STEPS
    bytes_per_launch = 16.0 * V + 28.0 * N
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_per_launch / in_graph / 1e9
    prof = profile_rows("k2d_step_batched512")
    sm_mhz = clock_info.get("sm_mhz") or 2070.0
    issue = None
    if prof["warp_inst"]:
        slots = 152 * 4 * sm_mhz * 1e6 * in_graph
        issue = {"warp_inst_per_launch": int(prof["warp_inst"]),
                 "issue_slots_per_launch": int(slots), "frac": round(prof["warp_inst"] / slots, 4),
                 "formula": "warp instructions / (152 SMs x 4 schedulers x SM clock x in-graph "
                            "launch time)",
                 "source": "profiles/k2d_step_batched512.md (ncu, build " +
                           str(prof["build"]) + ")"}
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS)",
            "kernel": "k2d_step (one launch per vertex-slot class, together)",
            "in_graph_us": round(in_graph * 1e6, 2),
            "in_graph_how": "one call of 32 steps timed again (L2 flushed) at the tuned "
                            "rebuild period and at half of it: the difference per extra rebuild "
                            "is rebuild_us; (headline ms_per_step - its rebuilds) / 32 is the "
                            "step launches' time inside the graph",
            "rebuild_us": None if rebuild is None else round(rebuild * 1e6, 2),
            "call_retimed_ms": None if t_full is None else round(t_full * 1e3, 4),
            "back_to_back_us": round(back_to_back * 1e6, 2),
            "back_to_back_how": "a rebuild period of step launches queued back to back after a "
                                "rebuild, warm, without the graph (each launch forks the "
                                "vertex-slot classes over two streams by events)",
            "cold_single_launch_us": round(kern * 1e6, 2),
            "cold_frac": round(bytes_per_launch / kern / 1e9 / peak, 4),
            "bytes_per_launch": int(bytes_per_launch),
            "traffic": None if prof["traffic"] is None else int(prof["traffic"]),
            "traffic_source": "profiles/k2d_step_batched512.md (ncu dram__bytes_read.sum + "
                              "dram__bytes_write.sum of one launch, build " +
                              str(prof["build"]) + ")",
            "issue": issue}


def e2e_leg(b, timed, V, args):
    """End to end through the C ABI: pinned host in, stepped, pinned host
    out; the input is the batch's current (relaxed) state, so the device work
    per step matches the timed region."""
    import torch
    xy_now, _ = b.download()
    xy_pin = torch.from_numpy(np.ascontiguousarray(xy_now.reshape(-1))).pin_memory()
    out_pin = torch.empty_like(xy_pin).pin_memory()
    f_pin = torch.empty_like(xy_pin).pin_memory()
    e_iters = max(3, min(args.steps, 10))

    def e2e_once():
        b.upload_ptr(xy_pin.data_ptr())
        b.step(SIM_STEPS, DT)
        b.download_ptr(out_pin.data_ptr(), f_pin.data_ptr())

    e2e_once()
    # host wall time of the three calls (upload and download return only
    # after their copies complete), L2 flushed before each iteration
    tt = 0.0
    for _ in range(e_iters):
        timed.flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e2e_once()
        tt += time.perf_counter() - t1
    return {"value": round(V * SIM_STEPS * e_iters / tt, 1), "unit": UNIT,
            "h2d_bytes_per_step": int(8 * V), "d2h_bytes_per_step": int(16 * V),
            "path": "dpm2d_upload + dpm2d_step(32) + dpm2d_download, pinned host buffers"}


def same_sample_leg(ctx, timed, tissues, args):
    """The 32 tissues the reference arm times, alone as one batch."""
    ts = sweep_sample(tissues)
    b, _ = make_batch(ctx, ts)
    tuned = b.autotune(DT, trial_blocks=2, use_cache=True)
    for _ in range(3):
        b.step(SIM_STEPS, DT)
    it = max(3, args.steps)
    s = timed(it, lambda: b.step(SIM_STEPS, DT))
    return {"value": round(b.nverts * SIM_STEPS / s, 1), "unit": UNIT,
            "ms_per_step": round(s * 1e3, 4), "sample": sample_desc(tissues),
            "sim_steps_per_step": SIM_STEPS, "tuning": tuned}


def plain_c1(ctx, timed, geo, stages=125, relax=500, phi_start=0.6, dphi=0.002,
             final_relax=37500):
    """The plain single-system path on the 2D jamming protocol: 1,024
    bidisperse cells from packing fraction 0.6, compressed to 0.85 in steps
    of 0.002 (dpm2d_set_packing_fraction on the device), 500 relaxation
    steps per stage, then a final relaxation at 0.85: 100,000 steps, timed
    whole."""
    t = workload_c1(geo)
    b, _ = make_batch(ctx, t)
    tuned = b.autotune(DT, trial_blocks=2, use_cache=True)
    b.step(relax, DT)  # the stage's graphs are captured outside the timed run
    b.upload(t[0]["xy"])  # start over from the initial state

    def protocol():
        for k in range(1, stages + 1):
            b.set_packing_fraction(phi_start + k * dphi)
            b.step(relax, DT)
        b.step(final_relax, DT)

    secs, _ = timed.span(protocol)
    d = b.diagnostics()
    si = d["perimeter"] / np.sqrt(4.0 * np.pi * d["area"])
    steps = stages * relax + final_relax
    return {"value": round(b.nverts * steps / secs, 1), "unit": UNIT,
            "seconds": round(secs, 3), "sim_steps": steps,
            "final": {"packing_fraction": round(float(d["packing_fraction"][0]), 5),
                      "shape_index_median": round(float(np.median(si)), 5),
                      "shape_index_mean": round(float(d["shape_index"][0]), 5),
                      "cells_below_half_a0": int(np.sum(d["area"] < 0.5 * t[0]["a0"])),
                      "mean_energy": float(np.mean(d["energy"]))},
            "workload": "1 tissue, 1024 cells x 32 vertices, bidisperse r0 1.0/1.4, "
                        "calA0 ~ U[1.0,1.2], kb=0.01, ka=kl=kc=1, dt=0.005; packing fraction "
                        f"{phi_start} -> {phi_start + stages * dphi:.3f} in steps of {dphi} "
                        f"with {relax} relaxation steps each, then {final_relax} at the final "
                        f"packing fraction ({steps} steps, rescale on the device)",
            "tuning": tuned}


def plain_c0(ctx, timed, geo, steps=10000):
    """The reference's own CPU-runnable case: 16 cells x 32 vertices,
    10,000 steps, timed whole."""
    t = workload_c0(geo)
    b, _ = make_batch(ctx, t)
    tuned = b.autotune(DT, trial_blocks=2, use_cache=True)
    b.upload(t[0]["xy"])
    b.step(steps, DT)  # graphs captured outside the timed run
    b.upload(t[0]["xy"])
    secs, _ = timed.span(lambda: b.step(steps, DT))
    return {"value": round(b.nverts * steps / secs, 1), "unit": UNIT,
            "seconds": round(secs, 4), "sim_steps": steps,
            "workload": "1 tissue, 16 cells x 32 vertices, calA0=1, ka=kl=kc=1, kb=0, "
                        "packing fraction 0.6, uniform random centres, dt=0.005, 10,000 steps",
            "tuning": tuned}


def plain3d(ctx, timed, iters, steps=16, level=3):
    """The plain 3D monolayer: 256 icospheres at subdivision 3 (642 vertices,
    1,280 faces); at level 2, the reference's own mesh (162 vertices, 320
    faces), the only one the reference can run."""
    from opencl_dpm_gb300 import clDPM
    t = build_monolayer(clDPM, np.random.default_rng(3), 256, level)
    b = make_batch3d(ctx, [t])
    for _ in range(3):
        b.step(steps, DT3)
    secs = timed(iters, lambda: b.step(steps, DT3))
    return {"value": round(b.nverts * steps / secs, 1), "unit": UNIT,
            "ms_per_step": round(secs * 1e3, 4), "sim_steps_per_step": steps,
            "workload": f"1 monolayer, 256 cells x {t['nv']} vertices (icosphere subdivision "
                        f"{level}), jittered hexagonal lattice on z=0, " + C2_NOTE}


def workload_batched3d():
    """48 monolayers of N ~ U{8..64} cells at subdivision 3 (seeded)."""
    from opencl_dpm_gb300 import clDPM
    rng = np.random.default_rng(5)
    return [build_monolayer(clDPM, rng, int(rng.integers(8, 65)), 3) for _ in range(48)]


def batched3d(ctx, timed, iters, steps=16):
    """Many independent 3D monolayers in one batch: 48 tissues of N ~
    U{8..64} cells at subdivision 3, one launch per step for all of them."""
    ts = workload_batched3d()
    b = make_batch3d(ctx, ts)
    for _ in range(3):
        b.step(steps, DT3)
    secs = timed(iters, lambda: b.step(steps, DT3))
    return {"value": round(b.nverts * steps / secs, 1), "unit": UNIT,
            "ms_per_step": round(secs * 1e3, 4), "sim_steps_per_step": steps,
            "tissues": len(ts), "cells": int(sum(len(t["Kv"]) for t in ts)),
            "vertices": int(b.nverts),
            "workload": "48 monolayers, N ~ U{8..64} cells x 642 vertices (subdivision 3), "
                        + C2_NOTE + ", one batch"}


SEQ_HOW = ("the plain single-system path over the same tissues one after another: each "
           "tissue alone as its own batch (2D: autotuned; small tissues take the resident "
           "run), warmed, then timed without an L2 flush; the tissues' times are summed")


def sequential_2d(ctx, timed, tissues):
    """The batched sweep's tissues through the plain path, one at a time:
    the summed time of one 32-step call per tissue."""
    total = 0.0
    for t in tissues:
        b, _ = make_batch(ctx, [t])
        b.autotune(DT, trial_blocks=2, use_cache=True)
        b.step(SIM_STEPS, DT)
        total += timed(3, lambda: b.step(SIM_STEPS, DT), flush=False)
        b.close()
    V = sum(int(np.sum(t["nv"])) for t in tissues)
    return {"value": round(V * SIM_STEPS / total, 1), "unit": UNIT,
            "ms_per_step": round(total * 1e3, 4), "sim_steps_per_step": SIM_STEPS,
            "tissues": len(tissues), "how": SEQ_HOW}


def sequential_3d(ctx, timed, ts, steps=16):
    """The batched 3D leg's monolayers through the plain path, one at a time."""
    total = 0.0
    for t in ts:
        b = make_batch3d(ctx, [t])
        b.step(steps, DT3)
        total += timed(3, lambda: b.step(steps, DT3), flush=False)
        b.close()
    V = sum(len(t["Kv"]) * t["nv"] for t in ts)
    return {"value": round(V * steps / total, 1), "unit": UNIT,
            "ms_per_step": round(total * 1e3, 4), "sim_steps_per_step": steps,
            "tissues": len(ts), "how": SEQ_HOW}


def service_time_alone(ctx, timed, t, sample_steps=256):
    """Seconds per step of one served request's tissue alone on the plain
    path (a batch of its own, warmed, `sample_steps` steps timed)."""
    if t["dim"] == 2:
        b, _ = make_batch(ctx, [t])
        b.autotune(DT, trial_blocks=2, use_cache=True)
        b.step(SIM_STEPS, DT)
        s = timed(1, lambda: b.step(sample_steps, DT), flush=False)
    else:
        b = make_batch3d(ctx, [t])
        b.step(16, DT3)
        s = timed(1, lambda: b.step(sample_steps, DT3), flush=False)
    b.close()
    return s / sample_steps


def fcfs(arrival, service):
    """Completion times of requests served one at a time in arrival order."""
    done = np.zeros(len(arrival))
    free = 0.0
    for i in np.argsort(arrival, kind="stable"):
        free = max(free, arrival[i]) + service[i]
        done[i] = free
    return done


def steady_state_leg(ctx, timed, geo, total=20000):
    """The sweep's full 20,000-step run from its initial lattice, in calls of
    32 steps timed one by one (no L2 flush: a continuous run): rate over the
    first 640 steps, around steps 2,000 and 10,000, the last 640, and the
    whole run."""
    tissues = workload_batched(geo)
    b, _ = make_batch(ctx, tissues)
    b.autotune(DT, trial_blocks=2, use_cache=True)
    b.step(SIM_STEPS, DT)  # graphs captured outside the timed run
    b.upload(np.concatenate([t["xy"] for t in tissues]))
    import torch
    calls = total // SIM_STEPS
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(calls + 1)]
    with torch.cuda.stream(timed.stream):
        ev[0].record(timed.stream)
        for i in range(calls):
            b.step(SIM_STEPS, DT)
            ev[i + 1].record(timed.stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    ms = np.array([ev[i].elapsed_time(ev[i + 1]) for i in range(calls)])
    rate = lambda a, z: round(b.nverts * SIM_STEPS * (z - a) / (ms[a:z].sum() / 1e3), 1)
    w = 20
    return {"unit": UNIT, "sim_steps": calls * SIM_STEPS,
            "steps_0_640": rate(0, w), "steps_2000_2640": rate(62, 62 + w),
            "steps_10000_10640": rate(312, 312 + w), "last_640": rate(calls - w, calls),
            "whole_run": rate(0, calls), "rebuilds_fallback": b.stats()[1]}


def disperse_leg(ctx, tissues, geo):
    """Setup cost: the reference's dispersion of cell centres (bit-exact on
    the device, dpm_disperse) for every tissue of the batched workload in one
    launch, and for the 1,024-cell plain tissue; the host loop on a few
    64-cell tissues for comparison."""
    from opencl_dpm_gb300 import clDPM
    from opencl_dpm_gb300.abi import disperse

    def centres(ts, seed0):
        X, Y = [], []
        for k, t in enumerate(ts):
            x, y = clDPM.drand48_centres(seed0 + k, len(t["nv"]), float(t["L"]))
            X.append(np.asarray(x, np.float32))
            Y.append(np.asarray(y, np.float32))
        return np.concatenate(X), np.concatenate(Y)

    def run(ts, seed0):
        X, Y = centres(ts, seed0)
        t0 = time.perf_counter()
        _, _, it = disperse(ctx, [len(t["nv"]) for t in ts],
                            np.concatenate([t["r0"] for t in ts]), [t["L"] for t in ts], X, Y)
        return time.perf_counter() - t0, it

    batch_s, batch_it = run(tissues, 1)
    plain = workload_c1(geo)
    plain_s, plain_it = run(plain, 7)
    # host loop on the four tissues nearest 64 cells, and the device on the same
    near = sorted(range(len(tissues)), key=lambda k: abs(len(tissues[k]["nv"]) - 64))[:4]
    sample = [tissues[k] for k in near]
    t0 = time.perf_counter()
    host_it = [clDPM.relax_centres(list(map(float, t["r0"])), float(t["L"]), 100 + k, False)[2]
               for k, t in enumerate(sample)]
    host_s = time.perf_counter() - t0
    dev_s, dev_it = run(sample, 100)
    return {"batched_tissues": len(tissues), "batched_s": round(batch_s, 3),
            "batched_max_iterations": int(batch_it.max()),
            "plain_1024_s": round(plain_s, 3), "plain_1024_iterations": int(plain_it[0]),
            "host_sample": {"tissues": len(sample), "cells": [len(t["nv"]) for t in sample],
                            "host_s": round(host_s, 3), "device_s": round(dev_s, 3),
                            "iterations_equal": [int(a) for a in dev_it] == host_it},
            "note": "bit-exact with the reference's host loop; one thread block per tissue"}


# ---------------------------------------------------------------------------
# served mixed stream (continuous batching through dpm_serve_*)
# ---------------------------------------------------------------------------

SERVE_CHUNK = 256
# (slots, cells per slot) of the 2D pools (NV <= 32) and of the 3D pools per
# subdivision level; slot memory is small next to HBM, so the pools are sized
# for concurrency
POOLS_2D = [(48, 128), (32, 512), (24, 2048)]
POOLS_3D = [(8, 128), (8, 128)]  # two pools per mesh: their steps run side by side


def served_requests(seed, nreq):
    """70% 2D tissues drawn like the batched sweep with N ~ U{16..2048} and
    NV in {16, 32}; 30% 3D monolayers with N ~ U{8..128} at subdivision 2 or
    3; each runs U{1000..50000} steps."""
    from opencl_dpm_gb300 import clDPM
    geo = ProductGeometry()
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(nreq):
        if rng.random() < 0.7:
            n = int(rng.integers(16, 2049))
            nv = int(rng.choice([16, 32]))
            kb = float(10 ** rng.uniform(-3, -1))
            calA = rng.uniform(1.0, 1.3, n)
            phi = float(rng.uniform(0.6, 0.9))
            t = build_tissue(geo, rng, n, np.full(n, nv), calA, np.ones(n), kb, phi)
            t["dim"] = 2
            t["verts"] = int(t["nv"].sum())
        else:
            n = int(rng.integers(8, 129))
            t = build_monolayer(clDPM, rng, n, int(rng.choice([2, 3])))
            t["verts"] = n * t["nv"]
        t["steps"] = int(rng.integers(1000, 50001))
        reqs.append(t)
    return reqs


def make_server(ctx):
    from opencl_dpm_gb300 import clDPM
    from opencl_dpm_gb300.abi import Server
    srv = Server(ctx, hbm_budget_bytes=32 << 30, chunk_steps=SERVE_CHUNK)
    for slots, cells in POOLS_2D:
        srv.add_pool2d(slots, cells, 32, DT)
    for level in (2, 3):
        proto = clDPM.Cell3D([0.0, 0.0, 0.0], 1.0, 1.0, level)
        faces = np.asarray(proto.GetFaces(), np.uint32)
        for slots, cells in POOLS_3D:
            srv.add_pool3d(slots, cells, faces, int(proto.NV), DT3)
    return srv


def submit(srv, t, steps=None):
    steps = t["steps"] if steps is None else steps
    if t["dim"] == 2:
        return srv.submit2d(t["nv"], t["Ka"], t["Kl"], t["Kb"], t["a0"], t["l0"], t["r0"],
                            t["xy"], float(t["L"]), t["Kre"], t["Kat"], 1, steps, DT)
    return srv.submit3d(t["nv"], t["Kv"], t["Ka"], t["Ks"], t["v0"], t["a0"], t["l0"],
                        t["xyz"], float(t["L"]), t["Kre"], 1, steps, DT3, Kb=t["Kb"],
                        adh=t["adh"])


def served_capacity(ctx, seed, nreq=32, steps=2048):
    """Vertex-steps/s of the server saturated with the same request mix (all
    submitted at once, each for `steps` steps)."""
    srv = make_server(ctx)
    reqs = served_requests(seed, nreq)
    for t in reqs:
        submit(srv, t, steps)
    t0 = time.perf_counter()
    srv.drain()
    secs = time.perf_counter() - t0
    vs, _ = srv.stats()
    srv.close()
    return vs / secs


def run_served(ctx, timed, nreq, plain2d, plain3d, seed=77):
    """Seeded Poisson arrivals at 80% of the server's measured capacity for
    this request mix; latency = completion - arrival (host clock).  Beside
    it, the same requests at the same arrival times served one at a time on
    the plain path: each request's tissue alone, its per-step time over 256
    steps times its steps, queued first come first served."""
    reqs = served_requests(seed, nreq)
    cap = served_capacity(ctx, seed + 2)
    mean_vs = float(np.mean([t["verts"] * t["steps"] for t in reqs]))
    lam = 0.8 * cap / mean_vs
    rng = np.random.default_rng(seed + 1)
    arrival = np.cumsum(rng.exponential(1.0 / lam, size=nreq))
    arrival -= arrival[0]

    srv = make_server(ctx)
    pool_bytes = srv.pool_bytes()

    ids = [None] * nreq
    done_at = np.zeros(nreq)
    running = set()
    nxt = 0
    rounds = 0
    t0 = time.perf_counter()
    while nxt < nreq or running:
        now = time.perf_counter() - t0
        while nxt < nreq and arrival[nxt] <= now:
            ids[nxt] = submit(srv, reqs[nxt])
            running.add(nxt)
            nxt += 1
        if not running:
            time.sleep(max(0.0, arrival[nxt] - (time.perf_counter() - t0)))
            continue
        srv.step()
        rounds += 1
        tnow = time.perf_counter() - t0
        for i in list(running):
            if srv.status(ids[i]) == 2:
                done_at[i] = tnow
                running.discard(i)
                srv.forget(ids[i])
    makespan = float(done_at.max())
    lat = done_at - arrival
    vs, _ = srv.stats()
    srv.close()
    dims = np.array([t["dim"] for t in reqs])
    n2 = int(np.sum(dims == 2))
    slow = int(np.argmax(lat))
    vs2 = float(sum(t["verts"] * t["steps"] for t in reqs if t["dim"] == 2))
    vs3 = float(sum(t["verts"] * t["steps"] for t in reqs if t["dim"] == 3))

    def pct(x):
        return {"p50": round(float(np.percentile(x, 50)), 4),
                "p99": round(float(np.percentile(x, 99)), 4)} if len(x) else None

    per_step = np.array([service_time_alone(ctx, timed, t) for t in reqs])
    service = per_step * np.array([t["steps"] for t in reqs], np.float64)
    seq_done = fcfs(arrival, service)
    seq_makespan = float(seq_done.max())
    seq_lat = seq_done - arrival

    return {
        "value": round(vs / makespan, 1), "unit": UNIT,
        "by_dim": {"2d": {"value": round(vs2 / makespan, 1),
                          "over_plain_2d": round(vs2 / makespan / plain2d, 3)},
                   "3d": {"value": round(vs3 / makespan, 1),
                          "over_plain_3d": round(vs3 / makespan / plain3d, 3)},
                   "note": "each dimension's vertex-steps over the whole makespan (2D and 3D "
                           "requests share the GPU), against its own plain path"},
        "latency_s": {"p50": round(float(np.percentile(lat, 50)), 4),
                      "p99": round(float(np.percentile(lat, 99)), 4),
                      "max": round(float(lat.max()), 4),
                      "2d": pct(lat[dims == 2]), "3d": pct(lat[dims == 3]),
                      "slowest": {"dim": int(dims[slow]), "vertices": int(reqs[slow]["verts"]),
                                  "steps": int(reqs[slow]["steps"]),
                                  "latency_s": round(float(lat[slow]), 3)}},
        "requests": nreq, "requests_2d": n2, "requests_3d": nreq - n2,
        "vertex_steps": vs, "makespan_s": round(makespan, 3), "rounds": rounds,
        "arrival_rate_per_s": round(lam, 3),
        "capacity": round(cap, 1),
        "sequential": {
            "value": round(vs / seq_makespan, 1), "unit": UNIT,
            "makespan_s": round(seq_makespan, 3),
            "busy_s": round(float(service.sum()), 3),
            "latency_s": {"p50": round(float(np.percentile(seq_lat, 50)), 4),
                          "p99": round(float(np.percentile(seq_lat, 99)), 4)},
            "served_over_sequential": round(seq_makespan / makespan, 2),
            "capacity_over_sequential": round(cap / (vs / float(service.sum())), 2),
            "how": "the same requests and arrival times served one at a time, first come first "
                   "served, on the plain path: each request's tissue alone as its own batch, its "
                   "per-step time over 256 timed steps times its steps"},
        "load": "arrival rate = 80% of the capacity measured first: the same server saturated "
                "with 32 requests of this mix, 2,048 steps each",
        "pools": {"2d": [{"slots": s, "cells": c, "nv_max": 32} for s, c in POOLS_2D],
                  "3d": [{"slots": s, "cells": c} for s, c in POOLS_3D],
                  "bytes": pool_bytes, "chunk_steps": SERVE_CHUNK},
        "workload": "seeded Poisson arrivals; 70% 2D (N~U{16..2048}, NV in {16,32}, params as "
                    "the batched sweep, dt=0.005), 30% 3D monolayers (N~U{8..128}, subdivision "
                    "2 or 3, " + C2_NOTE + "); steps~U{1000..50000}",
    }


# ---------------------------------------------------------------------------
# CPU baselines and the reference arm (the oracle; baseline use only)
# ---------------------------------------------------------------------------

def oracle_states(tissues):
    from oracle.oracle import Tissue2DState
    return [Tissue2DState(nv=t["nv"], xy=t["xy"].copy(), Ka=t["Ka"], Kl=t["Kl"], Kb=t["Kb"],
                          a0=t["a0"], l0=t["l0"], r0=t["r0"], L=float(t["L"]), Kre=1.0, Kat=0.0)
            for t in tissues]


def timed_oracle_2d(states, steps_per_round, threads, budget_s, max_rounds=None):
    """Rounds of `steps_per_round` oracle steps over every state until the
    budget is spent (at least one round); returns (vertex-steps/s, steps)."""
    from oracle.oracle import Port
    P = Port()
    verts = sum(int(s.nv.sum()) for s in states)
    t0 = time.perf_counter()
    done = 0
    while True:
        for s in states:
            P.run2d(s, steps_per_round, DT, nthreads=threads)
        done += steps_per_round
        el = time.perf_counter() - t0
        if el >= budget_s or (max_rounds is not None and done >= max_rounds * steps_per_round):
            break
    return verts * done / el, done


def cpu_baseline(tissues, budget_s=10.0):
    """The sweep's sample (every 16th tissue) on all host cores."""
    cores = os.cpu_count() or 1
    rate, done = timed_oracle_2d(oracle_states(sweep_sample(tissues)), 1, cores, budget_s)
    return {"value": round(rate, 1), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{sample_desc(tissues)}, {done} steps, all-pairs reference algorithm, "
                      "OpenMP over cells"}


def cpu_baselines_plain(geo, budget_s=10.0):
    """The plain configurations on the host cores, single-thread and
    all-core (the oracle restatement: the reference's all-pairs algorithm)."""
    from oracle.oracle import Port, Tissue3DState
    from opencl_dpm_gb300 import clDPM
    cores = os.cpu_count() or 1
    out = {"kind": "port", "cores_all": cores}
    # 16 cells: every one of the 10,000 steps, on all cores and on one
    # (about 5 s single-threaded)
    c0 = oracle_states(workload_c0(geo))
    r_all, n_all = timed_oracle_2d([c0[0].copy()], 10000, cores, 0.0, max_rounds=1)
    r_one, n_one = timed_oracle_2d([c0[0].copy()], 10000, 1, 0.0, max_rounds=1)
    out["c0"] = {"all_cores": round(r_all, 1), "all_cores_steps": n_all,
                 "single_thread": round(r_one, 1), "single_thread_steps": n_one,
                 "sample": "16 cells x 32 vertices (the whole workload)"}
    # 1,024 cells at packing fraction 0.6 (the protocol's first stage)
    c1 = oracle_states(workload_c1(geo))
    r_all, n_all = timed_oracle_2d([c1[0].copy()], 1, cores, budget_s / 4)
    r_one, n_one = timed_oracle_2d([c1[0].copy()], 1, 1, budget_s / 8, max_rounds=1)
    out["c1"] = {"all_cores": round(r_all, 1), "all_cores_steps": n_all,
                 "single_thread": round(r_one, 1), "single_thread_steps": n_one,
                 "sample": "1024 cells x 32 vertices at packing fraction 0.6"}
    # 3D monolayer: all-pairs winding numbers at subdivision 3; 32 cells on
    # all cores, 8 single-thread (the all-pairs sum grows as cells squared)
    P = Port()
    res = {}
    for name, ncell, thr in (("all_cores", 32, cores), ("single_thread", 8, 1)):
        t = build_monolayer(clDPM, np.random.default_rng(3), ncell, 3)
        s = Tissue3DState(nv=t["nv"], faces=t["faces"], xyz=t["xyz"].copy(), Kv=t["Kv"],
                          Ka=t["Ka"], Ks=t["Ks"], v0=t["v0"], a0=t["a0"], l0=t["l0"],
                          L=float(t["L"]), Kre=1.0, pbc=1, Kb=t["Kb"], adh=t["adh"])
        t0 = time.perf_counter()
        P.run3d(s, 1, DT3, nthreads=thr)
        res[name] = round(s.xyz.shape[0] / (time.perf_counter() - t0), 1)
        res[name + "_cells"] = ncell
    # the variant the reference itself can run: subdivision 2 (162 vertices)
    for name, ncell, thr in (("sub2_all_cores", 128, cores), ("sub2_single_thread", 16, 1)):
        t = build_monolayer(clDPM, np.random.default_rng(4), ncell, 2)
        s = Tissue3DState(nv=t["nv"], faces=t["faces"], xyz=t["xyz"].copy(), Kv=t["Kv"],
                          Ka=t["Ka"], Ks=t["Ks"], v0=t["v0"], a0=t["a0"], l0=t["l0"],
                          L=float(t["L"]), Kre=1.0, pbc=1, Kb=t["Kb"], adh=t["adh"])
        t0 = time.perf_counter()
        P.run3d(s, 1, DT3, nthreads=thr)
        res[name] = round(s.xyz.shape[0] / (time.perf_counter() - t0), 1)
        res[name + "_cells"] = ncell
    out["c2"] = dict(res, steps=1,
                     sample="monolayers of 32 (all cores) and 8 (one thread) cells x 642 "
                            "vertices (subdivision 3), and of 128 and 16 cells x 162 vertices "
                            "(subdivision 2, the reference's own mesh), one step each; the "
                            "oracle's winding sum runs over all cell pairs, so a 256-cell "
                            "monolayer runs ~8x (subdivision 3) or ~2x (subdivision 2) slower "
                            "per vertex than these samples")
    return out


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm restated in
    C; the reference's own OpenCL path cannot run on this machine, and its
    CPU build needs its source tree) on the host cores, over the sweep's
    32-tissue sample, 32 simulation steps per benchmark step.  Its inputs come
    from the oracle's own geometry: nothing of the product is loaded."""
    tissues = workload_batched(OracleGeometry())
    sample = oracle_states(sweep_sample(tissues))
    from oracle.oracle import Port
    P = Port()
    cores = os.cpu_count() or 1
    verts = sum(int(s.nv.sum()) for s in sample)

    def one():
        for s in sample:
            P.run2d(s, SIM_STEPS, DT, nthreads=cores)

    for _ in range(args.warmup):
        one()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one()
    secs = time.perf_counter() - t0
    value = verts * SIM_STEPS * args.steps / secs
    desc = (f"{sample_desc(tissues)}, {SIM_STEPS} simulation steps per benchmark step, "
            "all-pairs reference algorithm, OpenMP over cells")
    ncells = sum(len(t["nv"]) for t in tissues)
    nverts = sum(int(t["nv"].sum()) for t in tissues)
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(secs / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded tissues; see config)",
            "config": sweep_config(len(tissues), ncells, nverts),
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": cores,
                             "threads": cores, "kind": "port",
                             "oracle": "oracle/dpm_oracle.c (the oracle restatement; "
                                       "oracle/_ref needs the reference tree)",
                             "sample": desc},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def run_profile(kind):
    """A profiling target: the workload is set up and warmed as in the
    benchmark, then the launches to capture run inside the NVTX range
    "profile" (ncu --nvtx --nvtx-include "profile/"): for "2d" one fused step
    of the batched sweep (one launch per vertex-slot class) after a fresh
    neighbour-list rebuild; for "3d" one step of the 256-cell monolayer, for
    "3d48" one step of the 48 monolayers of the batched 3D leg."""
    import torch
    from opencl_dpm_gb300.abi import Context
    ctx = Context(0)
    if kind == "2d":
        tissues = workload_batched(ProductGeometry())
        b, _ = make_batch(ctx, tissues)
        b.autotune(DT, trial_blocks=2, use_cache=True)
        for _ in range(5):
            b.step(SIM_STEPS, DT)
        b.rebuild_now()
        torch.cuda.nvtx.range_push("profile")
        b.step_kernel(DT)
        ctx.synchronize()
        torch.cuda.nvtx.range_pop()
    else:
        from opencl_dpm_gb300 import clDPM
        if kind == "3d48":
            rng = np.random.default_rng(5)
            ts = [build_monolayer(clDPM, rng, int(rng.integers(8, 65)), 3) for _ in range(48)]
        else:
            ts = [build_monolayer(clDPM, np.random.default_rng(3), 256, 3)]
        b = make_batch3d(ctx, ts)
        for _ in range(3):
            b.step(16, DT3)
        ctx.synchronize()
        torch.cuda.nvtx.range_push("profile")
        b.step(1, DT3)
        ctx.synchronize()
        torch.cuda.nvtx.range_pop()
    print(json.dumps({"profile": kind, "ok": True}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--serve-requests", type=int, default=64,
                    help="requests in the served mixed stream (0 skips it)")
    ap.add_argument("--profile", choices=["2d", "3d", "3d48"], default=None,
                    help="run only a profiling target (see run_profile)")
    args = ap.parse_args()
    if args.profile:
        run_profile(args.profile)
        return 0
    args.warmup = max(3, args.warmup)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)), flush=True)
        return 0

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    line = run_ours(args, rank, world, local_rank)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
