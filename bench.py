#!/usr/bin/env python3
"""Benchmark of the GB300 DPM step (one JSON line on stdout).

Workload (default, the batched 2D sweep): 512 independent tissues with
N ~ U{8..256} cells and NV ~ {16, 24, 32, 48} vertices per cell (one NV per
tissue), per-tissue kb ~ LogU[1e-3, 1e-1], calA0 ~ U[1.0, 1.3], true packing
fraction ~ U[0.6, 0.9] (phi0 = sqrt(phi)), ka = kl = kc = 1, r0 = 1,
dt = 0.005.  Cells start as the Cell2D constructor's regular polygons, centred
on a seeded, jittered square lattice of the tissue's periodic box (synthetic
data; the reference names no dataset).  All tissues step together in one
batch; each simulation step is one launch of the fused step kernel, and the
neighbour-list rebuild plus one rebuild period of steps (8, 16 or 32, chosen
with warps per block and the register variant by the project's autotuner,
dpm2d_autotune) are one captured CUDA graph.

One benchmark "step" is one dpm2d_step call of 32 simulation steps of the
whole batch.
L2 (129 MB) is flushed by writing 256 MB before every timed iteration,
outside the timed events.  value = vertices * simulation steps / time.

Also reported: the plain single-tissue path on 1,024 bidisperse cells
("plain"), the 3D monolayer of 256 cells ("plain3d") and 48 smaller
monolayers in one batch ("batched3d"), the reference's dispersion on the
device ("disperse"), the dominant kernel's roofline, the end-to-end rate through the C
ABI with pinned host buffers ("e2e"), the served mixed stream of 2D and 3D
requests through dpm_serve_* with p50/p99 latency ("served"), SM clocks
during the timed region and the CPU baseline (the oracle restatement of the
reference on the host cores).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--serve-requests R]
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
L2_FLUSH_BYTES = 256 << 20
WORKLOAD_SWEEP = ("batched 2D sweep: 512 tissues, N~U{8..256}, NV in {16,24,32,48}, "
                  "kb~LogU[1e-3,1e-1], calA0~U[1,1.3], phi~U[0.6,0.9], ka=kl=kc=1, r0=1, dt=0.005")


# ---------------------------------------------------------------------------
# workloads (built with the product's own host model, clDPM)
# ---------------------------------------------------------------------------

def lattice_centres(rng, n, L, jitter=0.1):
    m = int(math.ceil(math.sqrt(n)))
    sp = L / m
    sites = rng.permutation(m * m)[:n]
    ix, iy = sites % m, sites // m
    c = np.stack([(ix + 0.5) * sp, (iy + 0.5) * sp], axis=1)
    c += rng.uniform(-jitter * sp, jitter * sp, size=c.shape)
    return c.astype(np.float32)


def build_tissue(clDPM, rng, n, nv, calA, r0, Kb, phi):
    """One tissue: regular polygons at lattice centres; returns arrays."""
    proto = [clDPM.Cell2D(0.0, 0.0, float(calA[i]), int(nv[i]), float(r0[i])) for i in range(n)]
    T = clDPM.Tissue2D(proto, float(np.sqrt(phi)))
    L = T.L
    cen = lattice_centres(rng, n, L)
    xy, a0, l0 = [], [], []
    for i, p in enumerate(proto):
        v = np.asarray(p.Verts, np.float32) + cen[i]
        xy.append(v)
        a0.append(p.a0)
        l0.append(p.l0)
    return dict(nv=np.asarray(nv, np.uint32), xy=np.concatenate(xy), a0=np.float32(a0),
                l0=np.float32(l0), r0=np.asarray(r0, np.float32),
                Ka=np.ones(n, np.float32), Kl=np.ones(n, np.float32),
                Kb=np.full(n, Kb, np.float32), L=np.float32(L), Kre=1.0, Kat=0.0)


def workload_batched(seed=0, ntissues=512):
    from opencl_dpm_gb300 import clDPM
    rng = np.random.default_rng(seed)
    tissues = []
    for t in range(ntissues):
        n = int(rng.integers(8, 257))
        nv = int(rng.choice([16, 24, 32, 48]))
        kb = float(10 ** rng.uniform(-3, -1))
        calA = rng.uniform(1.0, 1.3, n)
        phi = float(rng.uniform(0.6, 0.9))
        tissues.append(build_tissue(clDPM, rng, n, np.full(n, nv), calA, np.ones(n), kb, phi))
    return tissues


def workload_plain(seed=1, n=1024):
    from opencl_dpm_gb300 import clDPM
    rng = np.random.default_rng(seed)
    r0 = rng.permutation(np.r_[np.full(n // 2, 1.0), np.full(n - n // 2, 1.4)])
    calA = rng.uniform(1.0, 1.2, n)
    return [build_tissue(clDPM, rng, n, np.full(n, 32), calA, r0, 0.01, 0.6)]


DT3 = 0.002  # 3D monolayer time step


def build_monolayer(clDPM, rng, n, level, r0=1.0, calA=1.05):
    """n icospheres (Cell3D ctor geometry) resting on z = 0, centres on a
    jittered hexagonal lattice (spacing 2 r0, jitter U[-0.1, 0.1]) in a
    periodic box; kv=1, ka=0.5, ks=0.1, kb=0.05, adhesion range 0.1."""
    proto = clDPM.Cell3D([0.0, 0.0, 0.0], calA, r0, level)
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
    a0 = np.full(n, proto.a0, np.float32)
    # the host model's rest edge: sqrt(double(4 a0)) / sqrt(3), 4 a0 in float
    l0 = (np.sqrt((np.float32(4.0) * a0).astype(np.float64)) / np.sqrt(3.0)).astype(np.float32)
    f = lambda v: np.full(n, v, np.float32)
    return dict(dim=3, nv=int(proto.NV), faces=faces, xyz=xyz, Kv=f(1.0), Ka=f(0.5), Ks=f(0.1),
                v0=f(proto.v0), a0=a0, l0=l0, Kb=f(0.05), adh=f(0.1), L=L, Kre=1.0,
                level=level)


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


def profiled_traffic(summary):
    """DRAM bytes (read + write) per launch from the committed ncu summary
    `profiles/<summary>.md` (its "traffic (read + write) per launch" row)."""
    p = os.path.join(ROOT, "profiles", summary + ".md")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("| traffic (read + write) per launch"):
                    v, unit = line.split("|")[2].split()
                    return float(v) * {"MB": 1e6, "GB": 1e9, "KB": 1e3}[unit]
    except (OSError, ValueError, KeyError, IndexError):
        pass
    return None


def launches_per_call(batch, sim_steps, period):
    """Kernel launches of one dpm2d_step(sim_steps): per rebuild period one
    bin-preparation launch, 3 launches per radix pass, one neighbour-list
    launch; one fused step launch per simulation step."""
    lb, _, _, _ = batch.bins()
    tbits = int(math.ceil(math.log2(batch.ntissues))) if batch.ntissues > 1 else 0
    passes = (lb + tbits + 7) // 8
    blocks = math.ceil(sim_steps / period)
    return blocks * (1 + 3 * passes + 1) + sim_steps


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


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args, rank, world, local_rank):
    import torch
    from opencl_dpm_gb300.abi import Context

    torch.cuda.set_device(local_rank)
    ctx = Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local_rank)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local_rank}")

    tissues = workload_batched(seed=1000 + rank)
    b, xy_host = make_batch(ctx, tissues)
    V, N = b.nverts, b.ncells
    tuned = b.autotune(DT, trial_blocks=2, use_cache=True)

    def timed(batch, iters, fn):
        total = 0.0
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(iters)]
        with torch.cuda.stream(stream):
            for i in range(iters):
                flush.zero_()
                ev[i][0].record(stream)
                fn()
                ev[i][1].record(stream)
        torch.cuda.synchronize()
        ctx.synchronize()
        for s, e in ev:
            total += s.elapsed_time(e)
        return total / 1e3

    for _ in range(max(3, args.warmup)):
        b.step(SIM_STEPS, DT)
    ctx.synchronize()

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    secs = timed(b, args.steps, lambda: b.step(SIM_STEPS, DT))
    clock_info = clocks.stop()
    torch.cuda.synchronize()
    secs, units = reduce_over_ranks(secs, float(V) * SIM_STEPS * args.steps, world,
                                    f"cuda:{local_rank}")
    value = units / secs
    ms_per_step = secs / args.steps * 1e3

    if rank != 0:
        return None

    # dominant kernel: the fused step, launched alone after a flush
    nk = 20
    kern = timed(b, nk, lambda: b.step_kernel(DT)) / nk
    bytes_per_launch = 16.0 * V + 28.0 * N
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_per_launch / kern / 1e9
    traffic = profiled_traffic("k2d_step_batched512")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS)",
                "kernel": "k2d_step", "kernel_us": round(kern * 1e6, 2),
                "bytes_per_launch": int(bytes_per_launch),
                "traffic": None if traffic is None else int(traffic)}

    # end to end through the C ABI: pinned host in, stepped, pinned host out;
    # the input is the batch's current (relaxed) state, so the device work
    # per step matches the timed region
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
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e2e_once()
        tt += time.perf_counter() - t1
    e2e = {"value": round(V * SIM_STEPS * e_iters / tt, 1), "unit": UNIT,
           "h2d_bytes_per_step": int(8 * V), "d2h_bytes_per_step": int(16 * V),
           "path": "dpm2d_upload + dpm2d_step(32) + dpm2d_download, pinned host buffers"}

    # plain single-tissue path (1,024 cells) for the batched/plain ratio
    pt = workload_plain()
    pb, _ = make_batch(ctx, pt)
    ptuned = pb.autotune(DT, trial_blocks=2, use_cache=True)
    for _ in range(3):
        pb.step(SIM_STEPS, DT)
    p_secs = timed(pb, max(3, args.steps), lambda: pb.step(SIM_STEPS, DT))
    plain = {"value": round(pb.nverts * SIM_STEPS * max(3, args.steps) / p_secs, 1),
             "unit": UNIT, "ms_per_step": round(p_secs / max(3, args.steps) * 1e3, 4),
             "workload": "1 tissue, 1024 cells x 32 vertices, bidisperse r0 1.0/1.4, "
                         "calA0 ~ U[1.0,1.2], kb=0.01, packing fraction 0.6 (static box)",
             "tuning": ptuned}

    p3 = plain3d(ctx, lambda n, fn: timed(None, n, fn), max(3, args.steps))
    b3 = batched3d(ctx, lambda n, fn: timed(None, n, fn), max(3, args.steps))
    b3["batched_over_plain"] = round(b3["value"] / p3["value"], 2)
    disp = disperse_leg(ctx, tissues)

    served = None
    if args.serve_requests > 0:
        served = run_served(ctx, args.serve_requests)

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded tissues; see config)",
        "config": {"workload": WORKLOAD_SWEEP,
                   "tissues": b.ntissues, "cells": N, "vertices": V,
                   "sim_steps_per_step": SIM_STEPS,
                   "l2": "256 MB written before every timed iteration (outside the events)",
                   "graph": "one CUDA graph replay per cell-list rebuild period",
                   "tuning": tuned},
        "gpu_launches": launches_per_call(b, SIM_STEPS, tuned["rebuild_period"]) * args.steps,
        "roofline": roofline, "e2e": e2e, "plain": plain,
        "batched_over_plain": round(value / world / plain["value"], 2),
        "plain3d": p3,
        "batched3d": b3,
        "disperse": disp,
        "served": served,
        "clocks": clock_info,
    }
    line["cpu_baseline"] = cpu_baseline(tissues, budget_s=args.cpu_budget)
    return line


# ---------------------------------------------------------------------------
# served mixed stream (continuous batching through dpm_serve_*)
# ---------------------------------------------------------------------------

SERVE_CHUNK = 256
# (slots, cells per slot) of the 2D pools (NV <= 32) and of the 3D pools per
# subdivision level; slot memory is small next to HBM, so the pools are sized
# for concurrency
POOLS_2D = [(48, 128), (32, 512), (24, 2048)]
POOLS_3D = [(16, 128)]


def served_requests(seed, nreq):
    """70% 2D tissues drawn like the batched sweep with N ~ U{16..2048} and
    NV in {16, 32}; 30% 3D monolayers with N ~ U{8..128} at subdivision 2 or
    3; each runs U{1000..50000} steps."""
    from opencl_dpm_gb300 import clDPM
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(nreq):
        if rng.random() < 0.7:
            n = int(rng.integers(16, 2049))
            nv = int(rng.choice([16, 32]))
            kb = float(10 ** rng.uniform(-3, -1))
            calA = rng.uniform(1.0, 1.3, n)
            phi = float(rng.uniform(0.6, 0.9))
            t = build_tissue(clDPM, rng, n, np.full(n, nv), calA, np.ones(n), kb, phi)
            t["dim"] = 2
            t["verts"] = int(t["nv"].sum())
        else:
            n = int(rng.integers(8, 129))
            t = build_monolayer(clDPM, rng, n, int(rng.choice([2, 3])))
            t["verts"] = n * t["nv"]
        t["steps"] = int(rng.integers(1000, 50001))
        reqs.append(t)
    return reqs


def plain3d(ctx, timed, iters, steps=16):
    """The plain 3D monolayer: 256 icospheres at subdivision 3 (642 vertices,
    1,280 faces), kv=1, ka=0.5, ks=0.1, kb=0.05, adhesion range 0.1,
    dt=0.002; `timed(iters, fn)` returns seconds for iters calls of fn."""
    from opencl_dpm_gb300 import clDPM
    from opencl_dpm_gb300.abi import Batch3D
    t = build_monolayer(clDPM, np.random.default_rng(3), 256, 3)
    b = Batch3D(ctx, [256], t["faces"], t["nv"])
    b.set_cells(t["Kv"], t["Ka"], t["Ks"], t["v0"], t["a0"], t["l0"], t["Kb"], t["adh"])
    b.set_tissues([t["L"]], 1.0, 1)
    b.upload(t["xyz"])
    for _ in range(3):
        b.step(steps, DT3)
    secs = timed(iters, lambda: b.step(steps, DT3))
    return {"value": round(b.nverts * steps * iters / secs, 1), "unit": UNIT,
            "ms_per_step": round(secs / iters * 1e3, 4), "sim_steps_per_step": steps,
            "workload": "1 monolayer, 256 cells x 642 vertices (icosphere subdivision 3), "
                        "jittered hexagonal lattice on z=0, kv=1 ka=0.5 ks=0.1 kb=0.05, "
                        "adhesion 0.1, dt=0.002"}


def batched3d(ctx, timed, iters, steps=16):
    """Many independent 3D monolayers in one batch: 48 tissues of N ~
    U{8..64} cells at subdivision 3 (kv=1, ka=0.5, ks=0.1, kb=0.05, adhesion
    0.1, dt=0.002), one launch per step for all of them."""
    from opencl_dpm_gb300 import clDPM
    from opencl_dpm_gb300.abi import Batch3D
    rng = np.random.default_rng(5)
    ts = [build_monolayer(clDPM, rng, int(rng.integers(8, 65)), 3) for _ in range(48)]
    cat = lambda k: np.concatenate([t[k] for t in ts])
    b = Batch3D(ctx, [len(t["Kv"]) for t in ts], ts[0]["faces"], ts[0]["nv"])
    b.set_cells(cat("Kv"), cat("Ka"), cat("Ks"), cat("v0"), cat("a0"), cat("l0"), cat("Kb"),
                cat("adh"))
    b.set_tissues([t["L"] for t in ts], 1.0, 1)
    b.upload(cat("xyz"))
    for _ in range(3):
        b.step(steps, DT3)
    secs = timed(iters, lambda: b.step(steps, DT3))
    return {"value": round(b.nverts * steps * iters / secs, 1), "unit": UNIT,
            "ms_per_step": round(secs / iters * 1e3, 4), "sim_steps_per_step": steps,
            "tissues": len(ts), "cells": int(sum(len(t["Kv"]) for t in ts)),
            "vertices": int(b.nverts),
            "workload": "48 monolayers, N ~ U{8..64} cells x 642 vertices (subdivision 3), "
                        "kv=1 ka=0.5 ks=0.1 kb=0.05, adhesion 0.1, dt=0.002, one batch"}


def disperse_leg(ctx, tissues):
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
    plain = workload_plain()
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


def make_server(ctx):
    from opencl_dpm_gb300 import clDPM
    from opencl_dpm_gb300.abi import Server
    srv = Server(ctx, hbm_budget_bytes=32 << 30, chunk_steps=SERVE_CHUNK)
    for slots, cells in POOLS_2D:
        srv.add_pool2d(slots, cells, 32, DT)
    for level in (2, 3):
        proto = clDPM.Cell3D([0.0, 0.0, 0.0], 1.05, 1.0, level)
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


def run_served(ctx, nreq, seed=77):
    """Seeded Poisson arrivals at 80% of the server's measured capacity for
    this request mix; latency = completion - arrival (host clock)."""
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
    n2 = sum(1 for t in reqs if t["dim"] == 2)
    dims = np.array([t["dim"] for t in reqs])
    slow = int(np.argmax(lat))

    def pct(x):
        return {"p50": round(float(np.percentile(x, 50)), 4),
                "p99": round(float(np.percentile(x, 99)), 4)} if len(x) else None

    return {
        "value": round(vs / makespan, 1), "unit": UNIT,
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
        "load": "arrival rate = 80% of the capacity measured first: the same server saturated "
                "with 32 requests of this mix, 2,048 steps each",
        "pools": {"2d": [{"slots": s, "cells": c, "nv_max": 32} for s, c in POOLS_2D],
                  "3d": [{"slots": s, "cells": c} for s, c in POOLS_3D],
                  "bytes": pool_bytes, "chunk_steps": SERVE_CHUNK},
        "workload": "seeded Poisson arrivals; 70% 2D (N~U{16..2048}, NV in {16,32}, params as "
                    "the batched sweep, dt=0.005), 30% 3D monolayers (N~U{8..128}, subdivision "
                    "2 or 3, kv=1 ka=0.5 ks=0.1 kb=0.05 adhesion 0.1, dt=0.002); "
                    "steps~U{1000..50000}",
    }


# ---------------------------------------------------------------------------
# CPU baseline and the reference arm (the oracle; test/baseline use only)
# ---------------------------------------------------------------------------

def oracle_states(tissues):
    from oracle.oracle import Tissue2DState
    return [Tissue2DState(nv=t["nv"], xy=t["xy"].copy(), Ka=t["Ka"], Kl=t["Kl"], Kb=t["Kb"],
                          a0=t["a0"], l0=t["l0"], r0=t["r0"], L=float(t["L"]), Kre=1.0, Kat=0.0)
            for t in tissues]


def cpu_sample(tissues, every=16):
    return tissues[::every]


def cpu_baseline(tissues, budget_s=10.0, steps=None):
    from oracle.oracle import Port
    P = Port()
    sample = oracle_states(cpu_sample(tissues))
    cores = os.cpu_count() or 1
    verts = sum(int(s.nv.sum()) for s in sample)
    t0 = time.perf_counter()
    done = 0
    while True:
        for s in sample:
            P.run2d(s, 1, DT, nthreads=cores)
        done += 1
        el = time.perf_counter() - t0
        if (steps is not None and done >= steps) or (steps is None and el >= budget_s):
            break
    return {"value": round(verts * done / el, 1), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(sample)} of {len(tissues)} tissues (every 16th, {verts} vertices), "
                      f"{done} steps, all-pairs reference algorithm, OpenMP over cells"}


def run_reference(args):
    tissues = workload_batched(seed=1000)
    from oracle.oracle import Port
    P = Port()
    sample = oracle_states(cpu_sample(tissues))
    cores = os.cpu_count() or 1
    verts = sum(int(s.nv.sum()) for s in sample)
    for _ in range(args.warmup):
        for s in sample:
            P.run2d(s, 1, DT, nthreads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in sample:
            P.run2d(s, 1, DT, nthreads=cores)
    secs = time.perf_counter() - t0
    value = verts * args.steps / secs
    desc = (f"{len(sample)} of {len(tissues)} tissues (every 16th, {verts} vertices), "
            f"one simulation step per benchmark step, all-pairs reference algorithm")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(secs / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded tissues)",
            "config": {"workload": WORKLOAD_SWEEP, "sample": desc},
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": desc},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--serve-requests", type=int, default=64,
                    help="requests in the served mixed stream (0 skips it)")
    args = ap.parse_args()
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
