#!/usr/bin/env python
"""Benchmark of the GB300 simpois fill: filled Mpx/s at a 1e-6 FP64 relative residual.

Workload (default): Poisson with guidance, one 2048 x 2048 x 3 float32 image
(128 Gaussians per channel), guidance f = div of the forward-difference
gradient of an independent field, 6 irregular blobs covering 15 % of the
pixels, seeded synthetic data; every channel solved to an FP64 relative
residual <= 1e-6 (the workload's own target is 1e-5; 1e-6 is stricter).

A step is one converged solve of the whole image (all channels batched in one
call).  ``value`` times it with the inputs resident in HBM; ``e2e`` times the
same solve through the C-ABI host entry point (simpois_solve) from pinned host
buffers, host-to-device and device-to-host copies included; ``plain`` times
the same channels solved one per call.  L2 is flushed (a 512 MiB write)
between timed steps.

``--impl reference`` times the CPU restatement of the reference's CG recipe
(``CG_EPS = rtol * ||b|| simpois -s 1 -c -1``) on the host cores instead.
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


def make_workload(name, rank):
    from imscript_gb300 import synth
    seed = 1000 * rank
    if name == "c1":
        inst = synth.config1(seed=seed, rtol=1e-6)
        return [inst], "poisson-guided-2048x2048x3 (6 blobs, 15% holes)"
    if name == "c1s":  # reduced size, for quick checks
        inst = synth.config1(seed=seed, size=512, rtol=1e-6)
        return [inst], "poisson-guided-512x512x3 (6 blobs, 15% holes)"
    if name == "c0":
        return [synth.config0(seed=seed)], "laplace-512x512x1 (disks, 20% holes)"
    if name == "c3":
        return synth.config3(seed=seed), "batched-256-uneven (64..1024 px, 5-60% holes)"
    if name == "c2":
        return [synth.config2(seed=seed)], "biharmonic-4096x4096x1 (1024^2 square + 200 scratches)"
    if name == "c2s":  # reduced size, for quick checks
        return [synth.config2(seed=seed, size=1024, hole=256, n_scratch=50)], \
            "biharmonic-1024x1024x1 (256^2 square + 50 scratches)"
    raise SystemExit(f"unknown workload {name}")


# ------------------------------------------------------------------ CPU baseline

def cpu_sample(insts, crop, max_crops, seed=0):
    """Crops of the workload's channels with their unknowns, for the CPU."""
    rng = np.random.default_rng(seed)
    out = []
    chans = [(inst, l) for inst in insts for l in range(inst.g.shape[0])]
    tries = 0
    while len(out) < max_crops and tries < 64 * max_crops:
        inst, l = chans[tries % len(chans)]
        tries += 1
        _, h, w = inst.g.shape
        y0 = int(rng.integers(0, max(1, h - crop + 1)))
        x0 = int(rng.integers(0, max(1, w - crop + 1)))
        g = inst.g[l, y0:y0 + crop, x0:x0 + crop]
        n = int(np.isnan(g).sum())
        if 0 < n < g.size:
            f = None if inst.f is None else inst.f[l, y0:y0 + crop, x0:x0 + crop]
            out.append((np.ascontiguousarray(g), None if f is None else np.ascontiguousarray(f),
                        0 if inst.tstep > 0 else 1, inst.rtol))
    return out


def cpu_time(sample, threads):
    """Run the oracle's restatement of the reference CG recipe on every crop
    (CG_EPS = rtol * ||b||, -s 1 -c -1), in parallel threads."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle

    oracle.lib()

    def one(item):
        g, f, kind, rtol = item
        bn = float(oracle.rhs_norm(g[None], None if f is None else f[None], kind)[0])
        out, it, _ = oracle.cg_extension(g, f, init=np.zeros_like(g), maxit=-1, kind=kind,
                                         cg_eps=rtol * bn)
        return int(np.isnan(g).sum()), it

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, sample))
    dt = time.perf_counter() - t0
    unk = sum(r[0] for r in res)
    return unk, dt, res


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


def cpu_baseline(insts, budget_s=20.0):
    threads = os.cpu_count() or 1
    crop = 384
    sample = cpu_sample(insts, crop, max_crops=threads)
    unk, dt, res = cpu_time(sample, threads)
    return {"value": unk / dt / 1e6, "unit": "filled Mpx/s", "cores": threads, "kind": "port",
            "sample": f"{len(sample)} crops of {crop}x{crop} px cut from the workload's channels "
                      f"({unk} unknowns), each solved by the CPU restatement of the reference CG "
                      f"to FP64 relative residual 1e-6, one crop per thread; {dt:.1f} s"}


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

def run_diff(args):
    """32 x 1024^2 guided Poisson fills: forward (converged fill) and backward
    (adjoint solve + scatter) through the torch.autograd.Function, timed with
    CUDA events; reports forward filled Mpx/s and the bwd/fwd time ratio."""
    import torch
    from imscript_gb300 import autograd as ag, synth
    n = 32 if args.size == 0 else max(1, args.size)
    insts, targets, guid = synth.config4(seed=0, n=n)
    dev = torch.device("cuda", 0)
    base = torch.stack([torch.from_numpy(np.nan_to_num(i.g[0], nan=0.0)) for i in insts]).to(dev)
    mask = torch.stack([torch.from_numpy(np.isnan(i.g[0])) for i in insts]).to(dev)
    gx = torch.stack([torch.from_numpy(x) for x, _ in guid]).to(dev)
    gy = torch.stack([torch.from_numpy(y) for _, y in guid]).to(dev)
    tgt = torch.stack([torch.from_numpy(t) for t in targets]).to(dev)
    unknowns = int(mask.sum().item())
    stream = torch.cuda.current_stream(dev)
    fwd_ms, bwd_ms = [], []
    for it in range(args.warmup + args.steps):
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
        if it >= args.warmup:
            fwd_ms.append(e0.elapsed_time(e1))
            bwd_ms.append(e1.elapsed_time(e2))
    f_ms, b_ms = sum(fwd_ms) / len(fwd_ms), sum(bwd_ms) / len(bwd_ms)
    print(json.dumps({"workload": f"differentiation {n}x1024x1024 guided Poisson (MSE loss)",
                      "forward_ms": f_ms, "backward_ms": b_ms, "bwd_fwd_ratio": b_ms / f_ms,
                      "forward_filled_mpx_s": unknowns / (f_ms / 1e3) / 1e6,
                      "unknown_samples": unknowns, "steps": args.steps, "warmup": args.warmup}))


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
    if args.shard and world > 1:
        # one batch partitioned across the ranks (strong scaling), no collective
        # on the data path
        insts, wname = make_workload(args.workload, 0)
        insts = sdist.shard(insts, [i.unknowns for i in insts], rank, world)
        wname += f" sharded over {world} ranks"
    else:
        # every rank solves its own seeded copy of the workload (weak scaling)
        insts, wname = make_workload(args.workload, rank)
    unknowns = sum(i.unknowns for i in insts)
    gs = [torch.from_numpy(i.g).to(dev) for i in insts]
    fs = [None if i.f is None else torch.from_numpy(i.f).to(dev) for i in insts]
    outs = [torch.empty_like(g) for g in gs]
    rtol = insts[0].rtol
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    ctx = simpois.context(local, stream.cuda_stream)

    def step_batched():
        if len(insts) == 1:
            _, reps = simpois.solve(gs[0], fs[0], tstep=insts[0].tstep, rtol=rtol, out=outs[0])
        else:
            _, reps = simpois.solve_batch(list(zip(gs, fs, [i.tstep for i in insts])), rtol=rtol,
                                          outs=outs)
        return reps

    def step_plain():
        reps = []
        for g, f, i, o in zip(gs, fs, insts, outs):
            for l in range(g.shape[0]):
                _, r = simpois.solve(g[l:l + 1], None if f is None else f[l:l + 1], tstep=i.tstep,
                                     rtol=rtol, out=o[l:l + 1])
                reps += r
        return reps

    def barrier():
        if world > 1:
            dist.barrier()

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        reps = None
        barrier()
        torch.cuda.synchronize()
        for k in range(steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            reps = fn()
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        return ms, reps

    # untimed: the autotuner times the fused V-cycle's hand-over sizes on this
    # workload and the timed solves reuse its choice (the same output bits
    # whichever size it picks)
    coarse_max = None
    if not args.no_autotune:
        _, _, coarse_max = simpois.autotune(list(zip(gs, fs, [i.tstep for i in insts])), rtol=rtol,
                                            outs=outs)
    for _ in range(args.warmup):
        step_batched()
    ctx.reset_launches()
    with ClockSampler(local) as clocks:
        ms, reps = timed(step_batched, args.steps)
    launches = ctx.launches()
    bad = [r for r in reps if r["status"] not in (splib.OK,)]
    worst = max(r["rel_residual"] for r in reps)
    ms = sdist.max_over_ranks(ms, device=dev)
    total_unknowns = sdist.sum_over_ranks(unknowns, device=dev)
    value = total_unknowns * args.steps / (ms / 1e3) / 1e6
    if args.quick:
        line = {"value": value, "ms_per_step": ms / args.steps, "gpu_launches": launches,
                "iterations": [r["iterations"] for r in reps], "max_rel": worst,
                "coarse_max": coarse_max}
        if args.with_plain:
            step_plain()
            ms_p, _ = timed(step_plain, args.steps)
            line["plain_value"] = unknowns * args.steps / (ms_p / 1e3) / 1e6
            line["batched_over_plain"] = value / line["plain_value"]
        if rank == 0:
            print(json.dumps(line))
        return

    # kernel roofline: one more step of the same workload on the same stream,
    # launches issued eagerly with a CUDA-event pair around each main-loop
    # kernel; achieved = algorithmic bytes / event-timed duration
    ctx.reset_kernel_stats()
    flush.fill_(0.0)
    if len(insts) == 1:
        simpois.solve(gs[0], fs[0], tstep=insts[0].tstep, rtol=rtol, out=outs[0], flags=splib.FLAG_KTIMER)
    else:
        simpois.solve_batch(list(zip(gs, fs, [i.tstep for i in insts])), rtol=rtol, outs=outs,
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
        if args.workload == "c1":
            tr = ncu_traffic(dom, "poisson_guided_2048x2048x3")
            if tr:
                roofline.update(tr)

    # plain: one channel per call
    for _ in range(max(1, args.warmup // 2)):
        step_plain()
    ms_plain, reps_plain = timed(step_plain, args.steps)
    value_plain = unknowns * args.steps / (ms_plain / 1e3) / 1e6

    # e2e: the C-ABI host entry point, pinned host buffers
    e2e = None
    if len(insts) == 1:
        hg = torch.from_numpy(insts[0].g).pin_memory()
        hf = None if insts[0].f is None else torch.from_numpy(insts[0].f).pin_memory()
        ho = torch.empty_like(hg).pin_memory()
        hin = (hg.numpy(), None if hf is None else hf.numpy(), ho.numpy())

        def step_e2e():
            _, r = simpois.poisson_solver_separable(hin[0], hin[1], insts[0].tstep, rtol=rtol, out=hin[2])
            return r

        step_e2e()
        ms_e2e, _ = timed(step_e2e, args.steps)
        # page-locked, aligned buffers whose size is a multiple of 4 take the
        # direct path: g in; f only in the 4-pixel groups that hold an unknown;
        # out back whole during the solve, then its groups with an unknown
        g0 = insts[0].g
        direct = g0.size % 4 == 0 and os.environ.get("SIMPOIS_NO_DIRECT_IO", "0") in ("", "0")
        if direct:
            grp = int(np.isnan(g0.reshape(-1, 4)).any(axis=1).sum())
            bi = g0.nbytes + (0 if hf is None else 16 * grp)
            bo = g0.nbytes + 16 * grp
        else:
            bi = hg.numel() * 4 + (0 if hf is None else hf.numel() * 4)
            bo = ho.numel() * 4
        e2e = {"value": unknowns * args.steps / (ms_e2e / 1e3) / 1e6, "unit": "filled Mpx/s",
               "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo,
               "io": "direct" if direct else "copies", "ms_per_step": ms_e2e / args.steps}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    src = peak_src
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(insts)
    line = {
        "metric": "filled Mpx/s at 1e-6 rel. residual (FP64), batched vs plain on 1 GB300",
        "value": round(value, 3),
        "unit": "filled Mpx/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "strong" if (args.shard and world > 1) else "weak",
        "vs_baseline": None,
        "dtype": "f32 (FP64 refinement and reductions)",
        "data": "synthetic (seeded; shapes and distributions of the benchmark workload)",
        "config": {"workload": wname, "unknown_samples_per_step": unknowns, "rtol": rtol,
                   "l2": "flushed between timed steps (512 MiB write)",
                   "autotuned": {"coarse_max": coarse_max},
                   "parallelism": ("shards" if args.shard else "replicas") if world > 1 else "single GPU"},
        "plain": {"value": round(value_plain, 3), "unit": "filled Mpx/s",
                  "ms_per_step": ms_plain / args.steps,
                  "batched_over_plain": round(value / world / value_plain, 3)},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "solver": {"max_rel_residual": worst, "iterations": [r["iterations"] for r in reps],
                   "refinements": [r["refinements"] for r in reps], "not_ok": len(bad)},
        "roofline": roofline,
        "kernels": kernels,
        "cpu_baseline": cpu,
        "peaks_source": src,
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    insts, wname = make_workload(args.workload, 0)
    threads = os.cpu_count() or 1
    sample = cpu_sample(insts, 384, max_crops=threads)
    for _ in range(min(args.warmup, 1)):
        cpu_time(sample[: max(1, len(sample) // 4)], threads)
    tot_unk, tot_t = 0, 0.0
    for _ in range(args.steps):
        unk, dt, _ = cpu_time(sample, threads)
        tot_unk += unk
        tot_t += dt
    v = tot_unk / tot_t / 1e6
    line = {
        "metric": "filled Mpx/s at 1e-6 rel. residual (FP64), batched vs plain on 1 GB300",
        "impl": "reference",
        "value": round(v, 3), "unit": "filled Mpx/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 CG vectors, f32 stencil (as the reference)",
        "data": "synthetic (seeded)",
        "config": {"workload": wname, "rtol": insts[0].rtol},
        "cpu_baseline": {"value": round(v, 3), "unit": "filled Mpx/s", "cores": threads, "kind": "port",
                         "sample": f"per step {len(sample)} crops of 384x384 px of the workload, the "
                                   "reference CG recipe (CG_EPS = rtol*||b||, -s 1 -c -1) in the "
                                   "oracle's bit-exact C restatement, one crop per host thread"},
        "e2e": {"value": round(v, 3), "unit": "filled Mpx/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c1")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the untimed autotuning solve (default hand-over size)")
    ap.add_argument("--size", type=int, default=0, help="c4: number of images (default 32)")
    ap.add_argument("--shard", action="store_true",
                    help="N>1: partition one batch across the ranks instead of one copy per rank")
    ap.add_argument("--with-plain", action="store_true", help="--quick: also time one image per call")
    ap.add_argument("--quick", action="store_true",
                    help="batched solves only, short JSON (for profiling runs)")
    args = ap.parse_args()
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
