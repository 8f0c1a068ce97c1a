#!/usr/bin/env python
"""Benchmark of the GB300 simpois fill: filled Mpx/s at a 1e-6 FP64 relative residual.

Workload (default, ``--workload c3``): 256 uneven instances -- sides drawn
log-uniform in [64, 1024] (non-square), 1 or 3 float32 channels, 5-60 % holes
as random disks, half Laplace, half guided Poisson -- every channel solved to
an FP64 relative residual <= 1e-6.  Seeded synthetic data stands in for
images; three input sets (different seeds: sizes, masks and fields) are
solved in rotation, one per step, so that no step reuses the previous step's
plan or solve graph.

A step is one converged solve of a whole input set (all instances batched in
one call).  ``value`` times it with the inputs resident in HBM; ``plain``
times the same images solved one image per call; ``same_input`` times the
batched solve of one input set repeated (plan and graph reused); ``e2e``
times the batched solve through the C-ABI host entry point
(simpois_solve_batch_host) from page-locked host buffers, every copy to and
from the device included; ``bwd_fwd`` is the backward / forward time of the
differentiation workload (32 x 1024^2 guided Poisson, MSE loss) through the
torch.autograd.Function.  L2 is flushed (a 512 MiB write) between timed steps.

``--impl reference`` times the CPU restatement of the reference's CG recipe
(``CG_EPS = rtol * ||b|| simpois -s 1 -c -1``, bit-exact with the reference
binary) on the host cores, on whole images of the same input sets.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK = 6800.0
METRIC = "filled Mpx/s at 1e-6 rel. residual (FP64), batched vs plain on 1 GB300"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": HBM_FALLBACK}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


WORKLOADS = {
    "c3": "batched-256-uneven (64..1024 px, 1 or 3 ch, 5-60% holes as disks, half Laplace, half guided Poisson)",
    "c1": "poisson-guided-2048x2048x3 (6 blobs, 15% holes)",
    "c1s": "poisson-guided-512x512x3 (6 blobs, 15% holes)",
    "c0": "laplace-512x512x1 (disks, 20% holes)",
    "c2": "biharmonic-4096x4096x1 (1024^2 square + 200 scratches)",
    "c2s": "biharmonic-1024x1024x1 (256^2 square + 50 scratches)",
}


def make_workload(name, seed):
    """The instances of workload `name` for one seed."""
    from imscript_gb300 import synth
    if name == "c1":
        return [synth.config1(seed=seed, rtol=1e-6)]
    if name == "c1s":  # reduced size, for quick checks
        return [synth.config1(seed=seed, size=512, rtol=1e-6)]
    if name == "c0":
        return [synth.config0(seed=seed)]
    if name == "c3":
        return synth.config3(seed=seed)
    if name == "c2":
        return [synth.config2(seed=seed)]
    if name == "c2s":  # reduced size, for quick checks
        return [synth.config2(seed=seed, size=1024, hole=256, n_scratch=50)]
    raise SystemExit(f"unknown workload {name}")


def input_seeds(rank, rotate):
    """Seeds of the input sets a rank solves in rotation."""
    return [1000 * rank + k for k in range(max(1, rotate))]


def bench_config(args, sets):
    """The `config` of the line: the same dict on both arms."""
    unk = [sum(i.unknowns for i in insts) for insts in sets]
    return {"workload": WORKLOADS[args.workload], "instances_per_step": len(sets[0]),
            "unknown_samples_per_step": int(round(sum(unk) / len(unk))), "rtol": 1e-6,
            "inputs": f"{len(sets)} seeded input sets (sizes, masks and fields differ), one per step in rotation",
            "l2": "flushed between timed steps (512 MiB write)", "parallelism": "single GPU"}


# ------------------------------------------------------------------ CPU side

def _cg_channel(item):
    """The reference CG recipe (CG_EPS = rtol*||b||, -s 1 -c -1) on one whole
    channel, in the oracle's bit-exact C restatement."""
    from oracle import oracle
    g, f, kind, rtol = item
    bn = float(oracle.rhs_norm(g[None], None if f is None else f[None], kind)[0])
    out, it, _ = oracle.cg_extension(g, f, init=np.zeros_like(g), maxit=-1, kind=kind, cg_eps=rtol * bn)
    return int(np.isnan(g).sum()), it


def channels_of(insts):
    return [(np.ascontiguousarray(i.g[l]), None if i.f is None else np.ascontiguousarray(i.f[l]),
             0 if i.tstep > 0 else 1, i.rtol) for i in insts for l in range(i.g.shape[0])]


def cpu_time(chans, threads):
    """Solve every channel with the reference CG recipe, one channel per host
    thread at a time (the C code releases the GIL), largest first."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle
    oracle.lib()
    order = sorted(chans, key=lambda c: -int(np.isnan(c[0]).sum()))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(_cg_channel, order))
    dt = time.perf_counter() - t0
    return sum(r[0] for r in res), dt


def cpu_sample(insts, part, nparts):
    """Whole instances of the workload, every nparts-th one from `part`."""
    return [inst for k, inst in enumerate(insts) if k % nparts == part]


def cpu_baseline(insts, nparts):
    threads = os.cpu_count() or 1
    sub = cpu_sample(insts, 0, nparts)
    unk, dt = cpu_time(channels_of(sub), threads)
    return {"value": unk / dt / 1e6, "unit": "filled Mpx/s", "cores": threads, "kind": "port",
            "sample": f"{len(sub)} whole instances of the first input set (every {nparts}th, {unk} unknowns), "
                      f"each channel solved by the CPU restatement of the reference CG recipe to FP64 "
                      f"relative residual 1e-6, channels on {threads} host threads; {dt:.1f} s"}


def _fp64_err(item):
    """max |u - x| / max |x| over the filled pixels, x the FP64 direct solve"""
    from oracle import fp64
    g, f, kind, u = item
    x = fp64.solve(g, f, kind)
    m = np.isnan(g)
    if not m.any():
        return 0.0
    return float(np.abs(u[m].astype(np.float64) - x[m]).max() / max(np.abs(x[m]).max(), 1e-30))


def fp64_errors(insts, outs):
    """Error of every channel's output against the FP64 direct solve, in a
    process pool started with spawn (after CUDA is up a fork would hang)."""
    import multiprocessing as mp
    items = [(np.ascontiguousarray(i.g[l]), None if i.f is None else np.ascontiguousarray(i.f[l]),
              0 if i.tstep > 0 else 1, np.ascontiguousarray(o[l]))
             for i, o in zip(insts, outs) for l in range(i.g.shape[0])]
    items.sort(key=lambda it: -int(np.isnan(it[0]).sum()))
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        return pool.map(_fp64_err, items, chunksize=1)


def ncu_traffic(kernel, workload):
    """DRAM bytes (read + write) of the launch captured in the committed ncu
    summary profiles/<kernel>_<workload>.md, with the summary's title line
    and the algorithmic bytes it states for that launch; None when absent."""
    import re
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    tot = 0.0
    for key in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
        m = re.search(r"`%s`\) \| ([0-9.,]+) (\w+)" % re.escape(key), text)
        if not m:
            return None
        tot += float(m.group(1).replace(",", "")) * scale.get(m.group(2), 1.0)
    m = re.search(r"= ([0-9.]+) MB; DRAM traffic", text)
    return {"traffic": round(tot), "traffic_algorithmic": round(float(m.group(1)) * 1e6) if m else None,
            "traffic_source": f"profiles/{kernel}_{workload}.md ({text.splitlines()[0].lstrip('# ')}; "
                              "one launch, cold-cache ncu capture)"}


PROFILE_NAMES = {"c3": "batched_256_uneven", "c1": "poisson_guided_2048x2048x3"}


# ------------------------------------------------------------------ AMLE

def run_amle(args):
    """AMLE fill (imscript's amle, src/amle.c) of a 2048x2048x1 image with 20 %
    holes as disks, the reference's defaults AMLE_NN=4 and AMLE_NITER=100:
    filled Mpx/s (unknowns per second of the whole 100-iteration fill), inputs
    resident in HBM; e2e through the host entry point; the CPU baseline is the
    oracle's raster-order restatement (bit-exact with the reference binary) on
    a 512x512 crop, one thread like the reference."""
    import torch
    from imscript_gb300 import simpois, synth
    from oracle import oracle
    nn, niter = int(os.environ.get("AMLE_NN", 4)), 100
    rng = np.random.default_rng(77)
    size = 2048
    g = synth.gaussian_field(rng, size, size, 128)[None]
    g[:, synth.disk_mask(rng, size, size, 0.2, rmin=4, rmax=30)] = np.nan
    unknowns = int(np.isnan(g).sum())
    dev = torch.device("cuda", 0)
    gd = torch.from_numpy(g).to(dev)
    out = torch.empty_like(gd)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        simpois.amle(gd, nn=nn, niter=niter, out=out)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    actx = simpois.context(0, simpois._torch_stream(gd))
    actx.reset_launches()
    with ClockSampler(0) as clocks:
        for k in range(args.steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            _, gaps = simpois.amle(gd, nn=nn, niter=niter, out=out)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    launches = actx.launches() // args.steps
    # end to end: host buffers through simpois_amle, copies inside the timed region
    hin = torch.from_numpy(g).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    simpois.amle(hin.numpy(), nn=nn, niter=niter, out=hout.numpy())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        simpois.amle(hin.numpy(), nn=nn, niter=niter, out=hout.numpy())
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    # algorithmic bytes of the sweeps: per iteration and unknown, both iterates
    # read and written once (neighbour re-reads excluded) plus the mask byte
    alg = unknowns * niter * (2 * 4 + 2 * 4 + 1)
    peaks, peak_src = measured_peaks()
    peak = peaks.get("hbm_gbs")
    achieved = alg / (ms / 1e3) / 1e9
    traffic = ncu_traffic("k_amle_fused", f"amle_{size}x{size}x1") if nn == 4 else None
    if traffic:
        import re
        m = re.search(r"(\d+) iterations", traffic["traffic_source"])
        # the captured launch runs that many iterations out of shared memory:
        # its per-iteration algorithmic bytes (as `achieved` counts them) are
        # above the DRAM bytes it moves
        traffic["traffic_algorithmic"] = unknowns * int(m.group(1)) * (2 * 4 + 2 * 4 + 1) if m else None
    crop = g[:, :512, :512]
    t0 = time.perf_counter()
    oracle.amle(crop, nn=nn, niter=niter, order="raster")
    dt = time.perf_counter() - t0
    cu = int(np.isnan(crop).sum())
    line = {
        "metric": f"AMLE filled Mpx/s (AMLE_NN={nn}, AMLE_NITER={niter})",
        "value": round(unknowns / (ms / 1e3) / 1e6, 3), "unit": "filled Mpx/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Gaussian sum, disk holes)",
        "config": {"workload": f"amle-{size}x{size}x1 (disks, 20% holes)", "unknowns": unknowns,
                   "nn": nn, "niter": niter, "l2": "flushed between timed steps (512 MiB write)"},
        "e2e": {"value": unknowns / (e2e_ms / 1e3) / 1e6, "unit": "filled Mpx/s",
                "h2d_bytes_per_step": g.nbytes, "d2h_bytes_per_step": g.nbytes, "ms_per_step": e2e_ms},
        "gpu_launches": launches,
        "gap": {"max": gaps[0][0], "mean": gaps[0][1]},
        "clocks": clocks.summary(),
        "roofline": {"kernel": "k_amle_fused", "bound": "hbm", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if peak else None,
                     "traffic": None, "note": "whole call timed (init and output included)",
                     "peak_source": peak_src, **(traffic or {})},
        "cpu_baseline": {"value": cu / dt / 1e6, "unit": "filled Mpx/s", "cores": 1, "kind": "port",
                         "sample": f"512x512 crop ({cu} unknowns), raster-order restatement of "
                                   f"src/amle.c, {niter} iterations; {dt:.1f} s"},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ differentiation

def diff_times(steps, warmup, n=32):
    """n x 1024^2 guided Poisson fills (the differentiation workload): forward
    (converged fill) and backward (adjoint solve + scatter) through the
    torch.autograd.Function, timed with CUDA events; forward filled Mpx/s and
    the bwd/fwd time ratio."""
    import torch
    from imscript_gb300 import autograd as ag, synth
    insts, targets, guid = synth.config4(seed=0, n=n)
    dev = torch.device("cuda", torch.cuda.current_device())
    base = torch.stack([torch.from_numpy(np.nan_to_num(i.g[0], nan=0.0)) for i in insts]).to(dev)
    mask = torch.stack([torch.from_numpy(np.isnan(i.g[0])) for i in insts]).to(dev)
    gx = torch.stack([torch.from_numpy(x) for x, _ in guid]).to(dev)
    gy = torch.stack([torch.from_numpy(y) for _, y in guid]).to(dev)
    tgt = torch.stack([torch.from_numpy(t) for t in targets]).to(dev)
    unknowns = int(mask.sum().item())
    stream = torch.cuda.current_stream(dev)
    fwd_ms, bwd_ms = [], []
    for it in range(warmup + steps):
        img = base.clone().requires_grad_(True)
        Gx = gx.clone().requires_grad_(True)
        Gy = gy.clone().requires_grad_(True)
        g = torch.where(mask, torch.full_like(img, float("nan")), img)
        f = ag.divergence(Gx, Gy)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record(stream)
        u = ag.fill(g, f, rtol=1e-6)
        e1.record(stream)
        loss = 0.5 * ((u - tgt) ** 2).mean()
        loss.backward()
        e2.record(stream)
        torch.cuda.synchronize()
        if it >= warmup:
            fwd_ms.append(e0.elapsed_time(e1))
            bwd_ms.append(e1.elapsed_time(e2))
    f_ms, b_ms = sum(fwd_ms) / len(fwd_ms), sum(bwd_ms) / len(bwd_ms)
    return {"workload": f"differentiation {n}x1024x1024x1 guided Poisson, MSE loss, rtol 1e-6",
            "ratio": round(b_ms / f_ms, 3), "forward_ms": round(f_ms, 3), "backward_ms": round(b_ms, 3),
            "forward_filled_mpx_s": round(unknowns / (f_ms / 1e3) / 1e6, 1),
            "unknown_samples": unknowns, "steps": steps}


def run_diff(args):
    n = 32 if args.size == 0 else max(1, args.size)
    print(json.dumps(diff_times(args.steps, args.warmup, n)))


# ------------------------------------------------------------------ GPU arm

def run_ours(args):
    import torch
    import torch.distributed as dist
    from imscript_gb300 import simpois
    from imscript_gb300 import lib as splib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from imscript_gb300 import dist as sdist
    seeds = input_seeds(0 if args.shard else rank, args.rotate)
    sets = [make_workload(args.workload, sd) for sd in seeds]
    if args.shard and world > 1:
        # one batch partitioned across the ranks (strong scaling), no collective
        # on the data path
        sets = [sdist.shard(insts, [i.unknowns for i in insts], rank, world) for insts in sets]
    unk = [sum(i.unknowns for i in insts) for insts in sets]
    dsets = []
    for insts in sets:
        gs = [torch.from_numpy(i.g).to(dev) for i in insts]
        fs = [None if i.f is None else torch.from_numpy(i.f).to(dev) for i in insts]
        dsets.append((insts, gs, fs, [torch.empty_like(g) for g in gs]))
    rtol = 1e-6
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    ctx = simpois.context(local, stream.cuda_stream)

    def batched(k):
        insts, gs, fs, outs = dsets[k % len(dsets)]
        if len(insts) == 1:
            _, reps = simpois.solve(gs[0], fs[0], tstep=insts[0].tstep, rtol=rtol, out=outs[0])
        else:
            _, reps = simpois.solve_batch(list(zip(gs, fs, [i.tstep for i in insts])), rtol=rtol, outs=outs)
        return reps

    def plain(k):
        insts, gs, fs, outs = dsets[k % len(dsets)]
        reps = []
        for g, f, i, o in zip(gs, fs, insts, outs):
            _, r = simpois.solve(g, f, tstep=i.tstep, rtol=rtol, out=o)
            reps += r
        return reps

    def barrier():
        if world > 1:
            dist.barrier()

    def timed(fn, steps, same=False):
        """device time of `steps` steps (step k solves input set k, or set 0
        when `same`), CUDA events on the solve's stream, L2 flushed between"""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        reps = []
        barrier()
        torch.cuda.synchronize()
        for k in range(steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            reps.append(fn(0 if same else k))
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        units = sum(unk[0 if same else k % len(unk)] for k in range(steps))
        return ms, units, reps

    # untimed: the autotuner times the fused V-cycle's hand-over sizes and
    # sweeps per side on every input set, and the timed solves reuse its
    # choice (every choice meets the tolerance)
    tuned = None
    if not args.no_autotune:
        tuned = []
        for insts, gs, fs, outs in dsets:
            _, _, tn = simpois.autotune(list(zip(gs, fs, [i.tstep for i in insts])), rtol=rtol, outs=outs)
            tuned.append(tn)
    for k in range(args.warmup):
        batched(k)
    ctx.reset_launches()
    with ClockSampler(local) as clocks:
        ms, units, reps_all = timed(batched, args.steps)
    launches = ctx.launches()
    reps = [r for rs in reps_all for r in rs]
    bad = [r for r in reps if r["status"] != splib.OK]
    worst = max(r["rel_residual"] for r in reps)
    ms = sdist.max_over_ranks(ms, device=dev)
    units = sdist.sum_over_ranks(units, device=dev)
    value = units / (ms / 1e3) / 1e6
    if args.quick:
        line = {"value": value, "ms_per_step": ms / args.steps, "gpu_launches": launches,
                "iterations_max": max(r["iterations"] for r in reps), "max_rel": worst, "coarse_max": tuned}
        if args.with_plain:
            plain(0)
            ms_p, u_p, _ = timed(plain, args.steps)
            line["plain_value"] = u_p / (ms_p / 1e3) / 1e6
            line["batched_over_plain"] = value / world / line["plain_value"]
        if rank == 0:
            print(json.dumps(line))
        return

    # the same input set every step: the plan and the solve graph are reused
    ms_same, u_same, _ = timed(batched, args.steps, same=True)
    value_same = u_same / (ms_same / 1e3) / 1e6

    # kernel roofline: one more step of input set 0 on the same stream, the
    # launches issued eagerly with a CUDA-event pair around each main-loop
    # kernel; achieved = algorithmic bytes / event-timed duration
    ctx.reset_kernel_stats()
    flush.fill_(0.0)
    insts0, gs0, fs0, outs0 = dsets[0]
    if len(insts0) == 1:
        simpois.solve(gs0[0], fs0[0], tstep=insts0[0].tstep, rtol=rtol, out=outs0[0], flags=splib.FLAG_KTIMER)
    else:
        simpois.solve_batch(list(zip(gs0, fs0, [i.tstep for i in insts0])), rtol=rtol, outs=outs0,
                            flags=splib.FLAG_KTIMER)
    torch.cuda.synchronize()
    kstats = ctx.kernel_stats()
    peaks, peak_src = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", HBM_FALLBACK))
    kernels = {}
    for name, k in kstats.items():
        gbs = k["bytes"] / (k["ms"] * 1e-3) / 1e9 if k["ms"] > 0 else 0.0
        kernels[name] = {"launches": k["launches"], "ms_total": round(k["ms"], 4),
                         "avg_us": round(1e3 * k["ms"] / max(1, k["launches"]), 2),
                         "bytes_per_launch": k["bytes"] / max(1, k["launches"]),
                         "achieved_gbs": round(gbs, 1)}
    roofline = None
    if kernels:
        dom = max(kernels, key=lambda n: kernels[n]["ms_total"])
        d = kernels[dom]
        roofline = {"kernel": dom, "bound": "hbm", "achieved": d["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                    "frac": round(d["achieved_gbs"] / hbm, 4), "traffic": None,
                    "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                    else "fallback 6.8 TB/s"}
        if args.workload in PROFILE_NAMES:
            tr = ncu_traffic(dom, PROFILE_NAMES[args.workload])
            if tr:
                roofline.update(tr)

    # plain: one image per call
    for k in range(args.warmup):   # every input set once, as for the batched steps
        plain(k)
    ms_plain, u_plain, _ = timed(plain, args.steps)
    value_plain = u_plain / (ms_plain / 1e3) / 1e6

    # e2e: the C-ABI host entry point from page-locked host buffers, every
    # copy to and from the device inside the timed region
    hsets = []
    for insts, _, _, _ in dsets:
        hg = [torch.from_numpy(i.g).pin_memory() for i in insts]
        hf = [None if i.f is None else torch.from_numpy(i.f).pin_memory() for i in insts]
        ho = [torch.empty_like(g).pin_memory() for g in hg]
        hsets.append(([(g.numpy(), None if f is None else f.numpy(), i.tstep) for g, f, i in zip(hg, hf, insts)],
                      [o.numpy() for o in ho], (hg, hf, ho)))

    def e2e_step(k):
        items, houts, _ = hsets[k % len(hsets)]
        _, r = simpois.solve_batch_host(items, rtol=rtol, outs=houts, device=local)
        return r

    for k in range(args.warmup):   # as for the device-timed steps: every input set once
        e2e_step(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    e2e_ms = (time.perf_counter() - t0) * 1e3
    e2e_units = sum(unk[k % len(unk)] for k in range(args.steps))
    def moved(items, houts):
        """bytes in and out of one step: an image whose size is a multiple of 4
        (page-locked buffers) moves g whole, f and the output's unknown pixels
        in the 4-pixel groups that hold an unknown, the output whole during
        the solve; the others whole-buffer copies"""
        bi = bo = 0
        for (g, f, _), o in zip(items, houts):
            bi += g.nbytes
            bo += o.nbytes
            if g.size % 4 == 0:
                grp = 16 * int(np.isnan(g.reshape(-1, 4)).any(axis=1).sum())
                bi += 0 if f is None else grp
                bo += grp
            else:
                bi += 0 if f is None else f.nbytes
        return bi, bo

    io = [moved(hs[0], hs[1]) for hs in hsets]
    e2e = {"value": e2e_units / (e2e_ms / 1e3) / 1e6, "unit": "filled Mpx/s",
           "h2d_bytes_per_step": int(sum(b[0] for b in io) / len(io)),
           "d2h_bytes_per_step": int(sum(b[1] for b in io) / len(io)), "ms_per_step": e2e_ms / args.steps,
           "api": "simpois_solve_batch_host (page-locked buffers), wall clock"}

    # differentiation workload: bwd/fwd
    bwd_fwd = None
    if not args.no_diff and world == 1:
        bwd_fwd = diff_times(max(3, args.steps // 4), 2)

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    # after every timed region: the CPU baseline and the error against the
    # FP64 direct solve (host processes would disturb the timing)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(sets[0], args.cpu_parts)
    errs = None
    if not args.no_fp64_check:
        batched(0)
        torch.cuda.synchronize()
        errs = fp64_errors(sets[0], [o.cpu().numpy() for o in dsets[0][3]])
    line = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "filled Mpx/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "strong" if (args.shard and world > 1) else "weak",
        "vs_baseline": None,
        "dtype": "f32 (float-float refinement and dot products; FP64 Krylov vectors for the 13-point operator)",
        "data": "synthetic (seeded; shapes and distributions of the benchmark workload)",
        "config": bench_config(args, sets),
        "plain": {"value": round(value_plain, 3), "unit": "filled Mpx/s", "ms_per_step": ms_plain / args.steps,
                  "batched_over_plain": round(value / world / value_plain, 3), "calls": "one image per call"},
        "same_input": {"value": round(value_same, 3), "ms_per_step": ms_same / args.steps,
                       "note": "input set 0 every step: plan and solve graph reused"},
        "e2e": e2e,
        "bwd_fwd": bwd_fwd,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "autotuned": tuned,
        "solver": {"max_rel_residual": worst, "iterations_max": max(r["iterations"] for r in reps),
                   "refinements_max": max(r["refinements"] for r in reps), "not_ok": len(bad),
                   "max_err_vs_fp64": None if errs is None else max(errs),
                   "median_err_vs_fp64": None if errs is None else float(np.median(errs)),
                   "err_channels": None if errs is None else len(errs)},
        "roofline": roofline,
        "kernels": kernels,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_reference(args):
    """The reference CG recipe on the host cores: every step solves whole
    images -- every cpu_parts-th instance of one input set of the workload, the
    parts and the sets taken in rotation -- channels on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sets = [make_workload(args.workload, sd) for sd in input_seeds(0, args.rotate)]
    threads = os.cpu_count() or 1
    nparts = args.cpu_parts
    plan = [(k % len(sets), (k // len(sets)) % nparts) for k in range(args.steps)]
    if args.warmup:
        cpu_time(channels_of(cpu_sample(sets[0], nparts - 1, 4 * nparts)), threads)
    tot_unk, tot_t = 0, 0.0
    for si, part in plan:
        unk, dt = cpu_time(channels_of(cpu_sample(sets[si], part, nparts)), threads)
        tot_unk += unk
        tot_t += dt
    v = tot_unk / tot_t / 1e6
    line = {
        "metric": METRIC,
        "impl": "reference",
        "value": round(v, 3), "unit": "filled Mpx/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 CG vectors, f32 stencil (as the reference)",
        "data": "synthetic (seeded; shapes and distributions of the benchmark workload)",
        "config": bench_config(args, sets),
        "cpu_baseline": {"value": round(v, 3), "unit": "filled Mpx/s", "cores": threads, "kind": "port",
                         "sample": f"per step the whole images of every {nparts}th instance of one input set "
                                   f"(sets and parts in rotation), each channel solved by the reference CG "
                                   f"recipe (CG_EPS = rtol*||b||, -s 1 -c -1) in the oracle's bit-exact C "
                                   f"restatement, channels on {threads} host threads"},
        "e2e": {"value": round(v, 3), "unit": "filled Mpx/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1,
                    help="GPUs of the run (one process per GPU under torchrun; each solves its own input sets)")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c3")
    ap.add_argument("--rotate", type=int, default=3, help="input sets solved in rotation, one per step")
    ap.add_argument("--cpu-parts", type=int, default=2,
                    help="CPU legs: a step solves every n-th instance of an input set")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the error against the FP64 direct solve")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiation workload (bwd/fwd)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the untimed autotuning solves (default hand-over size)")
    ap.add_argument("--size", type=int, default=0, help="c4: number of images (default 32)")
    ap.add_argument("--shard", action="store_true",
                    help="N>1: partition one batch across the ranks instead of one copy per rank")
    ap.add_argument("--with-plain", action="store_true", help="--quick: also time one image per call")
    ap.add_argument("--quick", action="store_true",
                    help="batched solves only, short JSON (for profiling runs)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world and not (args.gpus == 1 and world == 1):
        if int(os.environ.get("RANK", "0")) == 0:
            print(f"bench: --gpus {args.gpus} but WORLD_SIZE {world}; launch N > 1 under torchrun",
                  file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c4":
        run_diff(args)
    elif args.workload == "amle":
        run_amle(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
